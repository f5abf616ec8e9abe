"""The split-BF16 tensor-core GEMM (tcgen05) against an FP64 product, for
every tile variant of the kernel and both product counts.

Split-BF16 products carry about 16 significant bits: the error of each entry is
bounded by ~3 * 2^-16 * sum_k |a_ik| |b_kj|, which the tests use as the scale.
With two products (A rounded to BF16) the bound is ~2^-8 of that scale.
"""
import ctypes

import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu


def variants():
    n = ctypes.c_int(0)
    sqbem.lib().sqbem_gemm_variants(ctypes.byref(n))
    return list(range(n.value))


def check(M, N, K, alpha=1.0, beta=0.0, seed=0, variant=-1, products=3):
    rng = np.random.default_rng(seed + M * 7 + N * 13 + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(K, N)).astype(np.float32)
    C = rng.normal(size=(M, N)).astype(np.float32)
    got = sqbem.gemm_mixed(A, B, C, alpha, beta, variant=variant, products=products)
    ref = alpha * (A.astype(np.float64) @ B.astype(np.float64)) + beta * C.astype(np.float64)
    scale = np.abs(alpha) * (np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64))) + abs(beta) * np.abs(C)
    err = np.max(np.abs(got - ref) / scale)
    assert err < (3e-5 if products == 3 else 6e-3), (M, N, K, variant, products, err)
    return err


SHAPES = [(128, 128, 64), (256, 128, 128), (128, 256, 192), (200, 300, 100), (1, 1, 1), (7, 130, 65),
          (1000, 37, 513), (513, 1025, 1000), (300, 520, 130)]


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_tc_gemm_shapes(M, N, K):
    check(M, N, K)


@pytest.mark.parametrize("products", [3, 2])
def test_tc_gemm_every_variant(products):
    """each tile variant (128 x 128 and 128 x 256 tiles) on ragged shapes, both
    product counts; the variant the autotuner picks must give the same error bound"""
    for v in variants():
        for (M, N, K) in SHAPES:
            check(M, N, K, variant=v, products=products)
        check(700, 900, 300, alpha=-1.0, beta=1.0, variant=v, products=products)


def test_tc_gemm_timing_entry_point():
    """sqbem_gemm_timing: device-resident grouped problems, seconds per launch"""
    for v in variants():
        t = ctypes.c_double(0)
        rc = sqbem.lib().sqbem_gemm_timing(v, 3, 512, 512, 512, 4, ctypes.c_float(1.0), 3, ctypes.byref(t))
        assert rc == sqbem.OK, sqbem.lib().sqbem_last_error()
        assert 0 < t.value < 1.0


def test_tc_gemm_alpha_beta():
    check(300, 200, 150, alpha=-1.0, beta=1.0)
    check(129, 257, 64, alpha=0.5, beta=-2.0)


def test_tc_gemm_large():
    """many tiles per CTA: exercises the persistent scheduler and both accumulators"""
    check(2048, 2048, 1024, alpha=-1.0, beta=1.0)
