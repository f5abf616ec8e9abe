"""GPU parity of the FP64 path (SQBEM_FP64) against the oracle and against
fixtures written by the reference itself (tests/golden/).

Bar: 1e-10 relative for every FP64 result (U, Omega, tractions, flux, field),
1e-13 for single panel integrals.  Relative errors of vectors are norm-wise:
max |x - x_ref| / max |x_ref|.
"""
import numpy as np
import pytest

from conftest import golden

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, float).reshape(-1), np.asarray(b, float).reshape(-1)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def uo_rel(sols, refs):
    """norm-wise relative error of the stacked (U, Omega) of all modes"""
    got = np.concatenate([np.concatenate([s.U, s.Om]) for s in sols])
    ref = np.concatenate([np.concatenate([np.asarray(r["U"]), np.asarray(r["Om"])]) for r in refs])
    return float(np.linalg.norm(got - ref) / np.linalg.norm(ref))


def test_panel_integrals_vs_reference(oracle):
    g = golden("panel")
    meshes = {"tube": sqbem.swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 12, 4),
              "sphere": sqbem.icosphere(1.0, 2, (0.7, 0, 0))}
    for k, m in meshes.items():
        ref = g[k]
        p = np.array(ref["p"], dtype=int)
        x0 = np.array(ref["x0"]).reshape(-1, 3)
        sf = np.array(ref["self"], dtype=np.int32)
        SL, DL = sqbem.panel_integrals(m.V[p], x0, sf)
        SLr = np.array(ref["SL"]).reshape(-1, 9)
        DLr = np.array(ref["DL"]).reshape(-1, 9)
        for i in range(len(p)):
            assert rel(SL[i], SLr[i]) < 1e-13, (k, i)
            if np.max(np.abs(DLr[i])) > 0:
                assert rel(DL[i], DLr[i]) < 1e-12, (k, i)
            else:
                assert np.max(np.abs(DL[i])) < 1e-15


def test_panel_integrals_random_vs_oracle(oracle):
    rng = np.random.default_rng(7)
    m = sqbem.icosphere(1.0, 3, (0.1, -0.2, 0.05))
    n = 4000
    p = rng.integers(0, m.P, n)
    # targets from just off the panel to far away: every rule is exercised
    d = np.exp(rng.uniform(np.log(0.05), np.log(20.0), n))
    x0 = m.centroid[p] + (d * m.h[p])[:, None] * rng.normal(size=(n, 3)) / np.sqrt(3)
    SL, DL = sqbem.panel_integrals(m.V[p], x0, 0)
    SLo, DLo = oracle.panel_integrals(m.V[p], x0, 0)
    err_s = np.max(np.abs(SL - SLo), axis=1) / np.max(np.abs(SLo), axis=1)
    # DL carries the factor r.m, which cancels for targets close to the panel's
    # plane; its error is measured against the kernel's own scale |SL| / dist.
    dist = np.linalg.norm(x0 - m.centroid[p], axis=1)
    scale_d = np.max(np.abs(DLo), axis=1) + np.max(np.abs(SLo), axis=1) / dist
    err_d = np.max(np.abs(DL - DLo), axis=1) / scale_d
    assert np.max(err_s) < 1e-12
    assert np.max(err_d) < 1e-11


def test_solve_dense_pivoting_and_singular():
    rng = np.random.default_rng(3)
    for n in (5, 64, 130, 301):
        A = rng.normal(size=(n, n))  # random: partial pivoting swaps rows
        B = rng.normal(size=(n, 3))
        X, piv = sqbem.solve_dense(A, B)
        assert piv
        assert rel(X, np.linalg.solve(A, B)) < 1e-9
        D = A + n * np.eye(n)  # diagonally dominant: no exchange, certified fast path
        X, piv = sqbem.solve_dense(D, B)
        assert not piv
        assert rel(X, np.linalg.solve(D, B)) < 1e-12
    S = rng.normal(size=(40, 40))
    S[:, 7] = 0.0  # exactly singular: zero pivot, as dgesv reports info > 0
    with pytest.raises(sqbem.BEMError) as e:
        sqbem.solve_dense(S, np.ones(40))
    assert e.value.code == sqbem.ERR_SINGULAR
    assert "dgesv failed" in str(e.value)


def kinematics(g, precision=sqbem.FP64, towed=True, field=True):
    a = 1.0
    lam, beta, nth, lev = g["a_over_R"], g["beta"], int(g["n_theta"]), int(g["sphere_level"])
    tube = sqbem.Tube(a / lam, g["L_over_R"] * a / lam, a, nth, precision=precision) if lam > 0 else None
    b = beta * (a / lam - a) if lam > 0 else 0.0
    s = sqbem.SwimmerSolver(tube, sqbem.icosphere(a, lev, (b, 0, 0)), (b, 0, 0), precision=precision)
    e = np.array(g["e"])
    sl1, sl2 = s.slip(e, 1, 0), s.slip(e, 0, 1)
    m = s.solve_free([sl1, sl2])
    out = {"B1": m[0], "B2": m[1], "s": s, "tube": tube}
    if towed and "towed_z" in g:
        out["towed_z"] = s.solve_prescribed((0, 0, 1), (0, 0, 0))
        out["drag_K"] = -s.force(out["towed_z"])[2] / (6 * np.pi)
        out["towed_gen"] = s.solve_prescribed((0.1, -0.2, 0.3), (0.05, 0.1, -0.15))
        out["force_gen"] = s.force(out["towed_gen"])
    if field and "points" in g:
        pts = np.array(g["points"]).reshape(-1, 3)
        out["vel_B1"] = s.velocity(m[0], sl1, pts)
        out["vel_B2"] = s.velocity(m[1], sl2, pts)
    return out


def check_solution(s, ref, tol):
    scale = max(np.linalg.norm(ref["U"]), np.linalg.norm(ref["Om"]), 1e-3)
    assert np.max(np.abs(s.U - ref["U"])) <= tol * scale
    assert np.max(np.abs(s.Om - ref["Om"])) <= tol * scale
    assert rel(s.f_sphere, ref["f_sphere"]) <= tol
    if ref["f_tube"]:
        assert rel(s.f_tube, ref["f_tube"]) <= tol


@pytest.mark.parametrize("case", ["offaxis", "tilted", "onaxis_l2", "unbounded"])
def test_swimmer_fp64_vs_reference(case):
    g = golden("swim_small")[case]
    o = kinematics(g)
    for k in ("B1", "B2", "towed_z", "towed_gen"):
        check_solution(o[k], g[k], FP64_TOL)
    assert abs(o["drag_K"] - g["drag_K"]) <= FP64_TOL * abs(g["drag_K"])
    assert rel(o["force_gen"], g["force_gen"]) <= FP64_TOL
    for k in ("vel_B1", "vel_B2"):
        assert rel(o[k], g[k]) <= FP64_TOL


def test_swimmer_fp64_vs_oracle_random(oracle):
    """seeded off-axis, tilted swimmer; every output against the oracle"""
    rng = np.random.default_rng(11)
    a, lam = 1.0, rng.uniform(0.2, 0.5)
    R = a / lam
    b = rng.uniform(0, 0.6) * (R - a)
    c = np.array([b * np.cos(0.3), b * np.sin(0.3), 0.0])
    e = rng.normal(size=3)
    e /= np.linalg.norm(e)
    t = sqbem.Tube(R, 4 * R, a, 10)
    s = sqbem.SwimmerSolver(t, sqbem.icosphere(a, 1, c), c)
    ot = oracle.Tube(R, 4 * R, a, 10)
    os_ = oracle.SwimmerSolver(ot, oracle.icosphere(a, 1, c), c)
    slips = [s.slip(e, 1, 0), s.slip(e, 0, 1), s.slip(e, 1.0, -2.5)]
    m = s.solve_free(slips)
    om = os_.solve_free([os_.slip(e, 1, 0), os_.slip(e, 0, 1), os_.slip(e, 1.0, -2.5)])
    for x, y in zip(m, om):
        assert rel(np.concatenate([x.U, x.Om]), np.concatenate([y.U, y.Om])) < FP64_TOL
        assert rel(x.f_sphere, y.f_sphere) < FP64_TOL
        assert rel(x.f_tube, y.f_tube) < FP64_TOL


def test_duct_fp64_vs_reference():
    g = golden("duct_small")
    d = sqbem.DuctFlow(1.0, 4.0, 8, 8, 3)
    assert d.mesh.P == g["P"]
    Q = [d.solve(dP, 0.0).Q for dP in g["dP"]]
    assert rel(Q, g["Q"]) < FP64_TOL
    s = d.solve(2.5, 0.5)
    assert abs(s.Q - g["Q_25_05"]) <= FP64_TOL * abs(g["Q_25_05"])
    assert rel(s.u, g["u"]) < FP64_TOL
    assert rel(s.f, g["f"]) < FP64_TOL
    v = d.velocity(d.solve(1.0, 0.0), np.array(g["points"]).reshape(-1, 3))
    assert rel(v, g["vel"]) < FP64_TOL


def test_duct_c1_fp64_vs_reference():
    """Full duct configuration: R = 1, L = 4, 24 x 24 x 6 (1680 panels)."""
    g = golden("duct_c1")
    d = sqbem.DuctFlow(1.0, 4.0, 24, 24, 6)
    assert d.mesh.P == 1680
    Q = np.array([d.solve(dP, 0.0).Q for dP in g["dP"]])
    assert rel(Q, g["Q"]) < FP64_TOL
    # outputs/duct_flow/flow_rate.csv of the reference (10 significant digits)
    np.testing.assert_allclose(Q, [0.04891121917, 0.09782243834, 0.1956448767, 0.3912897534], rtol=1e-9)
    s = d.solve(1.0, 0.0)
    assert rel(s.u, g["u1"]) < FP64_TOL
    assert rel(s.f, g["f1"]) < FP64_TOL
    v = d.velocity(s, np.array(g["points"]).reshape(-1, 3))
    assert rel(v, g["vel"]) < FP64_TOL


def test_level2_tube24_fp64_vs_reference():
    g = golden("c2_l2")
    for case in ("l2_axis", "l2_off", "l2_tilt"):
        o = kinematics(g[case])
        for k in ("B1", "B2"):
            check_solution(o[k], g[case][k], FP64_TOL)
        if "drag_K" in g[case]:
            assert abs(o["drag_K"] - g[case]["drag_K"]) <= FP64_TOL * g[case]["drag_K"]
        if "vel_B1" in g[case]:
            assert rel(o["vel_B1"], g[case]["vel_B1"]) < FP64_TOL


def test_c2_level3_fp64_vs_reference():
    """Full kinematics configuration (a/R = 0.3, level 3, n_theta = 24)."""
    g = golden("c2")["c2"]
    o = kinematics(g, field=False)
    for k in ("B1", "B2"):
        check_solution(o[k], g[k], FP64_TOL)
    assert abs(o["drag_K"] - g["drag_K"]) <= FP64_TOL * g["drag_K"]
    # outputs/reference/squirmer/axis.csv, a_over_R = 0.3 (10 significant digits)
    assert abs(o["drag_K"] - 2.369980169) < 1e-9
    assert abs(o["B1"].U[2] - 0.6313900133) < 1e-10
