"""Mixed-precision path (SQBEM_MIXED) against the FP64 reference.

Bar: U and Omega within 1e-6 relative of the FP64 oracle, measured norm-wise
over the stacked (U, Omega) of both squirming modes (the B2 mode on the axis is
~0, so a per-component relative error has no meaning there).  Tractions are
reported against 1e-5 (norm-wise, max-abs).  The refinement must reach its
1e-8 relative FP64 residual.
"""
import numpy as np
import pytest

from conftest import golden

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu

UO_TOL = 1e-6
F_TOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a, float).reshape(-1), np.asarray(b, float).reshape(-1)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def uo_rel(sols, refs):
    got = np.concatenate([np.concatenate([s.U, s.Om]) for s in sols])
    ref = np.concatenate([np.concatenate([np.asarray(r["U"]), np.asarray(r["Om"])]) for r in refs])
    return float(np.linalg.norm(got - ref) / np.linalg.norm(ref))


def mixed_kinematics(g, towed=True):
    a = 1.0
    lam, beta, nth, lev = g["a_over_R"], g["beta"], int(g["n_theta"]), int(g["sphere_level"])
    tube = sqbem.Tube(a / lam, g["L_over_R"] * a / lam, a, nth, precision=sqbem.MIXED) if lam > 0 else None
    b = beta * (a / lam - a) if lam > 0 else 0.0
    s = sqbem.SwimmerSolver(tube, sqbem.icosphere(a, lev, (b, 0, 0)), (b, 0, 0), precision=sqbem.MIXED)
    e = np.array(g["e"])
    m = s.solve_free([s.slip(e, 1, 0), s.slip(e, 0, 1)])
    it, res = s.refinement()
    out = {"B1": m[0], "B2": m[1], "it": it, "res": res, "s": s, "tube": tube}
    if towed and "towed_z" in g:
        out["towed_z"] = s.solve_prescribed((0, 0, 1), (0, 0, 0))
        out["drag_K"] = -s.force(out["towed_z"])[2] / (6 * np.pi)
    return out


@pytest.mark.parametrize("case", ["offaxis", "tilted", "onaxis_l2", "unbounded"])
def test_mixed_small_vs_reference(case):
    g = golden("swim_small")[case]
    o = mixed_kinematics(g)
    assert o["it"] >= 1 and o["res"] <= 1e-8
    err = uo_rel([o["B1"], o["B2"]], [g["B1"], g["B2"]])
    assert err < UO_TOL, err
    assert rel(o["B1"].f_sphere, g["B1"]["f_sphere"]) < F_TOL
    if g["B1"]["f_tube"]:
        assert rel(o["B1"].f_tube, g["B1"]["f_tube"]) < F_TOL
    assert abs(o["drag_K"] - g["drag_K"]) < UO_TOL * abs(g["drag_K"])
    assert rel(o["towed_z"].f_sphere, g["towed_z"]["f_sphere"]) < F_TOL


def test_mixed_level2_tube24_vs_reference():
    g = golden("c2_l2")
    for case in ("l2_axis", "l2_off", "l2_tilt"):
        o = mixed_kinematics(g[case], towed=False)
        err = uo_rel([o["B1"], o["B2"]], [g[case]["B1"], g[case]["B2"]])
        assert err < UO_TOL, (case, err)
        assert rel(o["B1"].f_tube, g[case]["B1"]["f_tube"]) < F_TOL, case


def test_mixed_c2_level3_vs_reference():
    """Full kinematics configuration: a/R = 0.3, level 3, n_theta = 24."""
    g = golden("c2")["c2"]
    o = mixed_kinematics(g)
    err = uo_rel([o["B1"], o["B2"]], [g["B1"], g["B2"]])
    assert err < UO_TOL, err
    assert abs(o["drag_K"] - g["drag_K"]) < UO_TOL * g["drag_K"]
    assert abs(o["B1"].U[2] - 0.6313900133) < 1e-6


def test_mixed_requires_mixed_tube():
    t = sqbem.Tube(10 / 3, 40 / 3, 1.0, 8, precision=sqbem.FP64)
    with pytest.raises(sqbem.BEMError) as e:
        sqbem.SwimmerSolver(t, sqbem.icosphere(1.0, 1), (0, 0, 0), precision=sqbem.MIXED)
    assert e.value.code == sqbem.ERR_ARG


def test_mixed_fp64_rsqrt_error_bound():
    """The FP64 reciprocal square root of the mixed path's near-singular and self
    integrals (an FP32 seed and one Newton step in FP64): relative error below
    2e-13 (1.5 e0^2 for the seed's e0 <= 2.7e-7) over the squared distances the
    integrals meet, and far beyond them."""
    import ctypes
    rng = np.random.default_rng(11)
    x = np.concatenate([10.0 ** rng.uniform(-8, 6, 200000), [1e-8, 1e-4, 0.25, 1.0, 2.0, 3.0, 1e6]])
    y = np.zeros_like(x)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert sqbem.lib().sqbem_test_rsqrt_nr(len(x), dp(x), dp(y)) == 0
    ref = 1.0 / np.sqrt(x)
    err = np.abs(y - ref) / ref
    assert err.max() < 2e-13, err.max()


@pytest.mark.parametrize("a_over_R,nth", [(0.3, 24), (0.6, 24), (0.1, 10)])
def test_tube_block_from_one_sector_matches_direct_assembly(a_over_R, nth):
    """the mixed path assembles the tube block from the rows of one sector and
    rotates 3 x 3 blocks (the mesh is n_theta-fold symmetric); against the
    direct FP32 assembly of every pair the entries differ by FP32 rounding only:
    1e-6 of the matrix's largest entry, and per panel pair 2e-6 of the largest
    entry of its 3 x 3 block (single entries of a block can cancel, so their own
    relative error is no measure)"""
    R = 1.0 / a_over_R
    Ts = sqbem.tube_block_f32(R, 4 * R, 1.0, nth, symmetric=True)
    Td = sqbem.tube_block_f32(R, 4 * R, 1.0, nth, symmetric=False)
    scale = float(np.max(np.abs(Td)))
    diff = np.abs(Ts.astype(np.float64) - Td)
    assert np.max(diff) <= 1e-6 * scale, np.max(diff) / scale
    n = Td.shape[0] // 3
    bd = diff.reshape(n, 3, n, 3).max(axis=(1, 3))
    bm = np.abs(Td.astype(np.float64)).reshape(n, 3, n, 3).max(axis=(1, 3))
    assert np.max(bd / bm) <= 2e-6, np.max(bd / bm)


@pytest.mark.parametrize("a_over_R,nth", [(0.3, 24), (0.6, 24), (0.1, 24), (0.3, 36), (0.3, 7)])
def test_tube_fourier_solve_inverts_the_tube_block(a_over_R, nth):
    """T^{-1} X through the tube's Fourier blocks (forward transform over the
    sectors, one tensor-core GEMM per frequency with the FP32 block inverses,
    inverse transform) against a dense FP64 solve with the same FP32 block T:
    within 1e-4 relative, the accuracy the refinement needs of its
    preconditioner (it stops at a 1e-8 residual either way)"""
    R = 1.0 / a_over_R
    T = sqbem.tube_block_f32(R, 4 * R, 1.0, nth, symmetric=True).astype(np.float64)
    rng = np.random.default_rng(nth)
    X = rng.normal(size=(T.shape[0], 5))
    Y = sqbem.tube_fourier_solve(R, 4 * R, 1.0, nth, X)
    ref = np.linalg.solve(T, X)
    err = np.linalg.norm(Y - ref) / np.linalg.norm(ref)
    res = np.linalg.norm(T @ Y - X) / np.linalg.norm(X)
    assert err <= 1e-4 and res <= 1e-4, (err, res)
