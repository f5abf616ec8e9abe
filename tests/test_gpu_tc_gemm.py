"""The split-BF16 tensor-core GEMM (tcgen05) against an FP64 product.

Split-BF16 products carry about 16 significant bits: the error of each entry is
bounded by ~3 * 2^-16 * sum_k |a_ik| |b_kj|, which the tests use as the scale.
"""
import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu


def check(M, N, K, alpha=1.0, beta=0.0, seed=0):
    rng = np.random.default_rng(seed + M * 7 + N * 13 + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(K, N)).astype(np.float32)
    C = rng.normal(size=(M, N)).astype(np.float32)
    got = sqbem.gemm_mixed(A, B, C, alpha, beta)
    ref = alpha * (A.astype(np.float64) @ B.astype(np.float64)) + beta * C.astype(np.float64)
    scale = np.abs(alpha) * (np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64))) + abs(beta) * np.abs(C)
    err = np.max(np.abs(got - ref) / scale)
    assert err < 3e-5, (M, N, K, err)
    return err


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 128, 128), (128, 256, 192), (200, 300, 100),
                                   (1, 1, 1), (7, 130, 65), (1000, 37, 513), (513, 1025, 1000)])
def test_tc_gemm_shapes(M, N, K):
    check(M, N, K)


def test_tc_gemm_alpha_beta():
    check(300, 200, 150, alpha=-1.0, beta=1.0)
    check(129, 257, 64, alpha=0.5, beta=-2.0)


def test_tc_gemm_large():
    """many tiles per CTA: exercises the persistent scheduler and both accumulators"""
    check(2048, 2048, 1024, alpha=-1.0, beta=1.0)
