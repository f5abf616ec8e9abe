"""The mixed far kernel's quadrature-rule decision (far_kernel_f32 in
assemble.cu), checked on the CPU.

The kernel forms the squared centroid distance in FP32 from hi + lo float pairs
and compares it with the squared thresholds (0.75 h)^2, (1.5 h)^2, (3 h)^2,
each widened to a +-1e-5 band. Only pairs inside a band take the exact FP64 test
of kernels.hpp:74-75.

This test emulates that arithmetic with numpy float32 (round to nearest) on the
meshes of sweep instances, built by the oracle. It asserts two things: no pair
decided in FP32 gets a rule other than the reference's FP64 decision, and
almost every pair is decided without FP64. The GPU may fuse the squared-distance
sum into multiply-adds; that only shrinks the rounding error the margin covers.
"""
import numpy as np
import pytest

from sqbem import workloads

f32 = np.float32
BAND = 1e-5


def _split(v):
    hi = v.astype(f32)
    return hi, (v - hi.astype(np.float64)).astype(f32)


def band_rule(ct, cs, h):
    """rule per (target, source) pair, -1 where the exact FP64 test decides"""
    th, tl = _split(ct)
    sh, sl = _split(cs)
    d = [(sh[None, :, q] - th[:, None, q]) + (sl[None, :, q] - tl[:, None, q]) for q in range(3)]
    d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
    t = [0.5625 * h * h, 2.25 * h * h, 9.0 * h * h]
    lo = [(x * (1 - BAND)).astype(f32)[None, :] for x in t]
    hi = [(x * (1 + BAND)).astype(f32)[None, :] for x in t]
    r = np.full(d2.shape, -1)
    r[d2 > hi[2]] = 0
    r[(r < 0) & (d2 < lo[2]) & (d2 > hi[1])] = 1
    r[(r < 0) & (d2 < lo[1]) & (d2 > hi[0])] = 2
    r[(r < 0) & (d2 < lo[0])] = 3
    return r


def exact_rule(ct, cs, h):
    """kernels.hpp:74-75: d = |c - x0| / h with the reference's FP64 rounding"""
    dx = cs[None, :, 0] - ct[:, None, 0]
    dy = cs[None, :, 1] - ct[:, None, 1]
    dz = cs[None, :, 2] - ct[:, None, 2]
    d = np.sqrt((dx * dx + dy * dy) + dz * dz) / h[None, :]
    return np.where(d < 0.75, 3, np.where(d < 1.5, 2, np.where(d < 3.0, 1, 0)))


@pytest.mark.parametrize("k", [0, 4])  # sweep instances 0 (sphere level 3) and 4 (level 2)
def test_fp32_rule_bands_match_the_exact_rule(oracle, k):
    ins = workloads.sweep()[k]
    a = 1.0
    R = a / ins["a_over_R"]
    b = ins["beta"] * (R - a)
    T = oracle.swimmer_tube_mesh(R, ins["L_over_R"] * R, a, ins["n_theta"], ins["n_r"])
    S = oracle.icosphere(a, ins["sphere_level"], (b, 0.0, 0.0))
    pairs = fallback = 0
    for tgt, src in ((T, T), (S, S), (T, S), (S, T)):
        rb = band_rule(tgt.centroid, src.centroid, src.h)
        rx = exact_rule(tgt.centroid, src.centroid, src.h)
        decided = rb >= 0
        assert np.array_equal(rb[decided], rx[decided])
        pairs += rb.size
        fallback += int((~decided).sum())
    assert fallback <= 1e-5 * pairs + 2, (fallback, pairs)


def test_sphere_sphere_rules_are_translation_invariant(oracle):
    """The mixed path shares one sphere-sphere block (built around the sphere's
    centre) among all same-level instances of a call.  That holds only if the
    reference's FP64 rule decisions for the translated sphere of every sweep
    instance equal those of the centred sphere: checked here for every
    instance of the sweep workload."""
    a = 1.0
    base = {lev: oracle.icosphere(a, lev, (0.0, 0.0, 0.0)) for lev in (2, 3)}
    rules = {lev: exact_rule(S.centroid, S.centroid, S.h) for lev, S in base.items()}
    for ins in workloads.sweep():
        R = a / ins["a_over_R"]
        b = ins["beta"] * (R - a)
        S = oracle.icosphere(a, ins["sphere_level"], (b, 0.0, 0.0))
        assert np.array_equal(exact_rule(S.centroid, S.centroid, S.h), rules[ins["sphere_level"]])
