"""Pin the CPU oracle (oracle/) against fixtures written by the reference itself.

The fixtures in tests/golden/ come from oracle/_ref/ref_dump, built from the
reference's own headers (tests/golden/make_golden.py); the published CSVs of the
reference (outputs/reference/squirmer/axis.csv, outputs/duct_flow/flow_rate.csv)
are restated below as the 10-digit values they hold.
"""
import numpy as np
import pytest

from conftest import golden


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_mesh_bitwise(oracle):
    g = golden("mesh")
    cases = {
        "swimmer_tube": lambda: oracle.swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 12, 4),
        "swimmer_tube_24": lambda: oracle.swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 24, 4),
        "duct": lambda: oracle.tube_mesh(1.0, oracle.uniform_z(0, 4, 6), 8, 3),
        "ico2": lambda: oracle.icosphere(1.0, 2, (0.7, -0.1, 0.2)),
    }
    for k, fn in cases.items():
        m = fn()
        ref = g[k]
        assert m.P == len(ref["area"]), k
        np.testing.assert_array_equal(m.V.reshape(-1), np.array(ref["V"]), err_msg=k)
        np.testing.assert_array_equal(m.normal.reshape(-1), np.array(ref["normal"]), err_msg=k)
        np.testing.assert_array_equal(m.centroid.reshape(-1), np.array(ref["centroid"]), err_msg=k)
        np.testing.assert_array_equal(m.area, np.array(ref["area"]), err_msg=k)
        np.testing.assert_array_equal(m.h, np.array(ref["h"]), err_msg=k)
        np.testing.assert_array_equal(m.tags, np.array(ref["tags"]).astype(int), err_msg=k)
    m = oracle.icosphere(1.0, 1)
    m.translate((0.25, 0.5, -0.75))
    np.testing.assert_array_equal(m.V.reshape(-1), np.array(g["ico1_translated"]["V"]))


def test_panel_integrals(oracle):
    g = golden("panel")
    x, w = oracle.gauss_legendre01(10)
    np.testing.assert_array_equal(x, g["gl10_x"])
    np.testing.assert_array_equal(w, g["gl10_w"])
    meshes = {"tube": oracle.swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 12, 4),
              "sphere": oracle.icosphere(1.0, 2, (0.7, 0, 0))}
    rules_seen = set()
    for k, m in meshes.items():
        ref = g[k]
        p = np.array(ref["p"], dtype=int)
        x0 = np.array(ref["x0"]).reshape(-1, 3)
        sf = np.array(ref["self"], dtype=np.int32)
        SL, DL = oracle.panel_integrals(m.V[p], x0, sf)
        for i in range(len(p)):
            rules_seen.add(oracle.rule_of(m.V[p[i]], x0[i], sf[i]))
        np.testing.assert_allclose(SL.reshape(-1), ref["SL"], rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(DL.reshape(-1), ref["DL"], rtol=1e-14, atol=1e-15)
    assert rules_seen == {0, 1, 2, 3, 4}


def test_quadrature_rules(oracle):
    for lev, n in enumerate([7, 28, 112, 448]):
        L, W = oracle.quadrature_rule(lev)
        assert L.shape == (n, 3)
        assert abs(W.sum() - 1) < 1e-14
        np.testing.assert_allclose(L.sum(axis=1), 1.0, atol=1e-15)


def _check_solution(s, ref, tol):
    scale = max(np.linalg.norm(ref["U"]), np.linalg.norm(ref["Om"]), 1e-3)
    assert np.max(np.abs(s.U - ref["U"])) <= tol * scale
    assert np.max(np.abs(s.Om - ref["Om"])) <= tol * scale
    fs = np.array(ref["f_sphere"])
    assert rel(s.f_sphere.reshape(-1), fs) <= tol
    if ref["f_tube"]:
        assert rel(s.f_tube.reshape(-1), ref["f_tube"]) <= tol


def kin_oracle(oracle, g, towed=True, field=True):
    a = 1.0
    lam, beta, nth, lev = g["a_over_R"], g["beta"], int(g["n_theta"]), int(g["sphere_level"])
    tube = oracle.Tube(a / lam, g["L_over_R"] * a / lam, a, nth) if lam > 0 else None
    b = beta * (a / lam - a) if lam > 0 else 0.0
    s = oracle.SwimmerSolver(tube, oracle.icosphere(a, lev, (b, 0, 0)), (b, 0, 0))
    e = np.array(g["e"])
    sl1, sl2 = s.slip(e, 1, 0), s.slip(e, 0, 1)
    m = s.solve_free([sl1, sl2])
    out = {"B1": m[0], "B2": m[1], "solver": s, "sl": (sl1, sl2)}
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


@pytest.mark.parametrize("case", ["offaxis", "tilted", "onaxis_l2", "unbounded"])
def test_swimmer_small(oracle, case):
    g = golden("swim_small")[case]
    o = kin_oracle(oracle, g)
    for k in ("B1", "B2", "towed_z", "towed_gen"):
        _check_solution(o[k], g[k], 1e-11)
    assert abs(o["drag_K"] - g["drag_K"]) <= 1e-11 * abs(g["drag_K"])
    np.testing.assert_allclose(o["force_gen"], g["force_gen"], rtol=1e-11, atol=1e-12)
    for k in ("vel_B1", "vel_B2"):
        assert rel(o[k].reshape(-1), g[k]) <= 1e-11


def test_duct_small(oracle):
    g = golden("duct_small")
    d = oracle.DuctFlow(1.0, 4.0, 8, 8, 3)
    assert d.mesh.P == g["P"]
    Q = [d.solve(dP, 0.0).Q for dP in g["dP"]]
    np.testing.assert_allclose(Q, g["Q"], rtol=1e-12)
    s = d.solve(2.5, 0.5)
    assert abs(s.Q - g["Q_25_05"]) <= 1e-12 * abs(g["Q_25_05"])
    assert rel(s.u.reshape(-1), g["u"]) <= 1e-12
    assert rel(s.f.reshape(-1), g["f"]) <= 1e-12
    v = d.velocity(d.solve(1.0, 0.0), np.array(g["points"]).reshape(-1, 3))
    assert rel(v.reshape(-1), g["vel"]) <= 1e-12


def test_trajectory_small(oracle):
    g = golden("traj")
    P = oracle.TrajectoryParams(alpha=-1.5, a_over_R=0.3, beta0=0.5, pitch0_deg=5, yaw0_deg=10,
                                dt=0.5, t_max=3.0, n_theta=12, sphere_level=1)
    rows, status = oracle.run_trajectory(P)
    assert status == g["status"]
    lines = [l for l in g["csv"].split("\n") if l and not l.startswith("#") and not l.startswith("t,")]
    ref = np.array([[float(x) for x in l.split(",")] for l in lines])
    assert rows.shape == ref.shape
    # the CSV holds 10 significant digits
    np.testing.assert_allclose(rows, ref, rtol=2e-9, atol=1e-12)
    for r, l in zip(rows, lines):
        assert ",".join(oracle.fmt10(v) for v in r) == l


@pytest.mark.slow
def test_duct_c1_published(oracle):
    """Full duct configuration (24 x 24 x 6, 1680 panels) against the
    reference's dump and its published flow_rate.csv (10 digits)."""
    g = golden("duct_c1")
    d = oracle.DuctFlow(1.0, 4.0, 24, 24, 6)
    Q = np.array([d.solve(dP, 0.0).Q for dP in g["dP"]])
    np.testing.assert_allclose(Q, g["Q"], rtol=1e-12)
    published = [0.04891121917, 0.09782243834, 0.1956448767, 0.3912897534]
    np.testing.assert_allclose(Q, published, rtol=1e-9)
    v = d.velocity(d.solve(1.0, 0.0), np.array(g["points"]).reshape(-1, 3))
    assert rel(v.reshape(-1), g["vel"]) <= 1e-12


@pytest.mark.slow
def test_level2_tube24(oracle):
    g = golden("c2_l2")
    for case in ("l2_axis", "l2_off", "l2_tilt"):
        o = kin_oracle(oracle, g[case], towed=True, field=True)
        for k in ("B1", "B2"):
            _check_solution(o[k], g[case][k], 1e-10)
        if "drag_K" in g[case]:
            assert abs(o["drag_K"] - g[case]["drag_K"]) <= 1e-10 * g[case]["drag_K"]
        if "vel_B1" in g[case]:
            assert rel(o["vel_B1"].reshape(-1), g[case]["vel_B1"]) <= 1e-10


@pytest.mark.slow
def test_c2_published(oracle):
    """a/R = 0.3, beta = 0, level 3, n_theta = 24: the reference dump (17 digits)
    and its published axis.csv row (10 digits)."""
    g = golden("c2")["c2"]
    o = kin_oracle(oracle, g, towed=True, field=False)
    for k in ("B1", "B2"):
        _check_solution(o[k], g[k], 1e-10)
    assert abs(o["drag_K"] - g["drag_K"]) <= 1e-10 * g["drag_K"]
    # outputs/reference/squirmer/axis.csv, row a_over_R = 0.3
    assert abs(o["drag_K"] - 2.369980169) < 1e-9
    assert abs(o["B1"].U[2] - 0.6313900133) < 1e-10
