"""Trajectories (src/trajectory.hpp) on the GPU: the drop-in run_trajectory
against the reference's own CSV, checkpoint / resume, and the batched ensemble
against the oracle."""
import math
import os

import numpy as np
import pytest

from conftest import golden

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu

SMALL = dict(alpha=-1.5, a_over_R=0.3, beta0=0.5, pitch0_deg=5, yaw0_deg=10, dt=0.5, t_max=3.0, n_theta=12,
             sphere_level=1)


def read_csv(path):
    lines = open(path).read().splitlines()
    head = [l for l in lines if l.startswith("#") or l.startswith("t,")]
    rows = np.array([[float(x) for x in l.split(",")] for l in lines if l and l[0] not in "#t"])
    return head, rows


def golden_rows():
    g = golden("traj")
    lines = [l for l in g["csv"].split("\n") if l]
    head = [l for l in lines if l.startswith("#") or l.startswith("t,")]
    rows = np.array([[float(x) for x in l.split(",")] for l in lines if l[0] not in "#t"])
    return g["status"], head, rows


def test_run_trajectory_fp64_matches_reference_csv(tmp_path):
    status, head_ref, rows_ref = golden_rows()
    prefix = str(tmp_path / "traj_small")
    st = sqbem.run_trajectory(sqbem.TrajParams(**SMALL), prefix, precision=sqbem.FP64)
    assert st == status
    head, rows = read_csv(prefix + ".csv")
    assert head == head_ref  # comment and header lines byte-identical
    assert rows.shape == rows_ref.shape
    np.testing.assert_allclose(rows, rows_ref, rtol=2e-9, atol=1e-12)  # 10 printed digits
    assert not os.path.exists(prefix + ".ckpt")  # removed unless paused


def test_run_trajectory_mixed_within_1e6(tmp_path):
    _, _, rows_ref = golden_rows()
    prefix = str(tmp_path / "traj_mixed")
    sqbem.run_trajectory(sqbem.TrajParams(**SMALL), prefix, precision=sqbem.MIXED)
    _, rows = read_csv(prefix + ".csv")
    assert rows.shape == rows_ref.shape
    err = np.max(np.abs(rows - rows_ref)) / np.max(np.abs(rows_ref))
    assert err < 1e-6, err


def test_pause_and_resume_from_checkpoint(tmp_path):
    """budget_s tiny: the run pauses after its first step and keeps the
    checkpoint; the second call resumes from it and finishes like one run."""
    _, _, rows_ref = golden_rows()
    prefix = str(tmp_path / "traj_resume")
    st1 = sqbem.run_trajectory(sqbem.TrajParams(**SMALL, budget_s=1e-9), prefix, precision=sqbem.FP64)
    assert st1 == "paused"
    assert os.path.exists(prefix + ".ckpt")
    t, step, nh = open(prefix + ".ckpt").readline().split()
    assert float(t) == 0.5 and int(step) == 1 and int(nh) == 1
    st2 = sqbem.run_trajectory(sqbem.TrajParams(**SMALL), prefix, precision=sqbem.FP64)
    assert st2 == "finished"
    _, rows = read_csv(prefix + ".csv")
    np.testing.assert_allclose(rows, rows_ref, rtol=2e-9, atol=1e-12)


def _initial_states(P, n, rng):
    R = 1.0 / P.a_over_R
    y0 = []
    for k in range(n):
        b = rng.uniform(0.1, 0.6) * (R - 1.0)
        ph = rng.uniform(0, 2 * math.pi)
        e = rng.normal(size=3)
        e /= np.linalg.norm(e)
        y0.append([b * math.cos(ph), b * math.sin(ph), 0.0, *e])
    return np.array(y0)


def test_ensemble_fp64_matches_oracle(oracle):
    """three swimmers, the reference scheme (RK4 start-up + AB4), against the
    oracle's evaluation loop"""
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.5, n_theta=8, sphere_level=1)
    rng = np.random.default_rng(4)
    y0 = _initial_states(P, 3, rng)
    alpha = np.array([-2.0, 0.0, 3.0])
    steps = 5
    states, U, Om, status, _ = sqbem.trajectory_ensemble(y0, alpha, P, steps, scheme=0, precision=sqbem.FP64)
    assert np.all(status == 0)
    R = 1.0 / P.a_over_R
    tube = oracle.Tube(R, 4 * R, 1.0, 8)
    sph0 = oracle.icosphere(1.0, 1)

    def evaluate(y, al):
        c = np.array([y[0], y[1], 0.0])
        e = np.array(y[3:6]) / np.linalg.norm(y[3:6])
        S = sph0.copy()
        S.translate(c)
        s = oracle.SwimmerSolver(tube, S, c)
        k = s.solve_free([s.slip(e, 1, 0), s.slip(e, 0, 1)])
        u = k[0].U + al * k[1].U
        w = k[0].Om + al * k[1].Om
        return np.concatenate([u, np.cross(w, e)])

    for m in range(3):
        y = y0[m].copy()
        hist = []
        for s in range(steps):
            d = evaluate(y, alpha[m])
            if len(hist) < 3:
                k2 = evaluate(y + 0.25 * d, alpha[m])
                k3 = evaluate(y + 0.25 * k2, alpha[m])
                k4 = evaluate(y + 0.5 * k3, alpha[m])
                y = y + 0.5 / 6 * (d + 2 * k2 + 2 * k3 + k4)
            else:
                y = y + 0.5 / 24 * (55 * d - 59 * hist[2] + 37 * hist[1] - 9 * hist[0])
            y[3:6] /= np.linalg.norm(y[3:6])
            hist = (hist + [d])[-3:]
            np.testing.assert_allclose(states[m, s + 1], y, rtol=1e-9, atol=1e-11)


def test_ensemble_mixed_vs_fp64_rk4():
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.25, n_theta=10, sphere_level=1)
    rng = np.random.default_rng(9)
    y0 = _initial_states(P, 5, rng)
    alpha = rng.uniform(-5, 5, 5)
    s64, U64, _, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 4, scheme=1, precision=sqbem.FP64)
    smx, Umx, _, _, t = sqbem.trajectory_ensemble(y0, alpha, P, 4, scheme=1, precision=sqbem.MIXED)
    assert t > 0
    assert np.max(np.abs(smx - s64)) < 1e-6 * np.max(np.abs(s64))
    assert np.max(np.abs(Umx - U64)) < 1e-6 * np.max(np.abs(U64))


def test_ensemble_mixed_vs_fp64_config5_mesh():
    """the trajectory-ensemble workload's own mesh (a/R = 0.3, n_theta = 24,
    level 2, dt = 0.05): 8 of its swimmers, 4 RK4 steps, mixed against FP64"""
    from sqbem import workloads
    w = workloads.ensemble()[:8]
    P = sqbem.TrajParams(a_over_R=w[0]["a_over_R"], dt=w[0]["dt"], n_theta=w[0]["n_theta"],
                         sphere_level=w[0]["sphere_level"], L_over_R=w[0]["L_over_R"])
    R = 1.0 / P.a_over_R
    y0 = np.array([[d["beta0"] * (R - 1.0), 0.0, 0.0, *d["e"]] for d in w])
    alpha = np.array([d["alpha"] for d in w])
    s64, U64, O64, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 4, scheme=1, precision=sqbem.FP64)
    smx, Umx, Omx, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 4, scheme=1, precision=sqbem.MIXED)
    assert np.max(np.abs(smx - s64)) < 1e-6 * np.max(np.abs(s64))
    for k in range(len(w)):
        uo = np.concatenate([Umx[k].reshape(-1), Omx[k].reshape(-1)])
        ref = np.concatenate([U64[k].reshape(-1), O64[k].reshape(-1)])
        assert np.linalg.norm(uo - ref) < 1e-6 * np.linalg.norm(ref), k


def test_tube_factor_shared_across_calls():
    """two ensemble calls and a field call around the same tube assemble and
    factor it once (the cache of factored tubes); results are unchanged"""
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.25, n_theta=9, sphere_level=1)
    rng = np.random.default_rng(17)
    y0 = _initial_states(P, 3, rng)
    alpha = rng.uniform(-5, 5, 3)
    sqbem.tube_cache_clear()
    b0, h0, _ = sqbem.tube_cache_stats()
    s1, U1, _, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 2, scheme=1, precision=sqbem.MIXED)
    s2, U2, _, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 2, scheme=1, precision=sqbem.MIXED)
    sqbem.ensemble_field(s2[:, -1, :], alpha, P, 5, 5, 7, 7.0, precision=sqbem.MIXED)
    b1, h1, n = sqbem.tube_cache_stats()
    assert b1 - b0 == 1 and h1 - h0 == 2 and n >= 1
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(U1, U2)
    sqbem.tube_cache_clear()
    s3, _, _, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 2, scheme=1, precision=sqbem.MIXED)
    assert sqbem.tube_cache_stats()[0] - b1 == 1
    np.testing.assert_array_equal(s1, s3)


def test_ensemble_wall_contact_freezes_member():
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.5, n_theta=8, sphere_level=1, beta_stop=0.5)
    R = 1.0 / P.a_over_R
    y0 = np.array([[0.6 * (R - 1.0), 0, 0, 0, 0, 1.0], [0.1 * (R - 1.0), 0, 0, 0, 0, 1.0]])
    states, U, _, status, _ = sqbem.trajectory_ensemble(y0, [0.0, 0.0], P, 2, scheme=1, precision=sqbem.MIXED)
    assert status[0] == 1 and status[1] == 0
    np.testing.assert_array_equal(states[0, 2], y0[0])
    assert np.all(np.isnan(U[0]))


def _field_reference(P, y, alpha, pts, tube, precision=sqbem.FP64):
    """single-swimmer API: SwimmerSolver.velocity for the combined slip"""
    c = np.array([y[0], y[1], 0.0])
    e = np.array(y[3:6]) / np.linalg.norm(y[3:6])
    S = sqbem.icosphere(1.0, P.sphere_level, c)
    s = sqbem.SwimmerSolver(tube, S, c, precision=precision)
    slip = s.slip(e, 1.0, alpha)
    sol = s.solve_free([slip])[0]
    return s.velocity(sol, slip, pts)


def test_ensemble_field_fp64_matches_swimmer_velocity():
    P = sqbem.TrajParams(a_over_R=0.3, n_theta=10, sphere_level=1)
    R = 1.0 / P.a_over_R
    y = np.array([[0.5, -0.3, 2.0, 0.0, 0.6, 0.8], [-0.8, 0.2, 0.0, 1.0, 0.0, 0.0]])
    alpha = np.array([-2.0, 3.0])
    nx, ny, nz = 9, 8, 11
    u, secs = sqbem.ensemble_field(y, alpha, P, nx, ny, nz, 5.0, precision=sqbem.FP64)
    assert secs > 0 and u.shape == (2, nx, ny, nz, 3)
    tube = sqbem.Tube(R, P.L_over_R * R, 1.0, P.n_theta, 4)
    for k in range(2):
        pts, mask = sqbem.field_grid(R, (y[k, 0], y[k, 1], 0.0), nx, ny, nz, 5.0)
        uk = u[k].reshape(-1, 3)
        assert np.all(np.isnan(uk[~mask])) and not np.any(np.isnan(uk[mask]))
        ref = _field_reference(P, y[k], alpha[k], pts[mask], tube)
        err = np.max(np.abs(uk[mask] - ref)) / np.max(np.abs(ref))
        assert err < 1e-11, err


def test_ensemble_field_matches_oracle(oracle):
    P = sqbem.TrajParams(a_over_R=0.35, n_theta=8, sphere_level=1)
    R = 1.0 / P.a_over_R
    y = np.array([[0.4, 0.1, 0.0, 0.0, 0.0, 1.0]])
    u, _ = sqbem.ensemble_field(y, [1.5], P, 5, 5, 7, 4.0, precision=sqbem.FP64)
    pts, mask = sqbem.field_grid(R, (0.4, 0.1, 0.0), 5, 5, 7, 4.0)
    c = np.array([0.4, 0.1, 0.0])
    otube = oracle.Tube(R, P.L_over_R * R, 1.0, P.n_theta)
    s = oracle.SwimmerSolver(otube, oracle.icosphere(1.0, 1, c), c)
    slip = s.slip(np.array([0.0, 0.0, 1.0]), 1.0, 1.5)
    sol = s.solve_free([slip])[0]
    ref = s.velocity(sol, slip, pts[mask])
    err = np.max(np.abs(u[0].reshape(-1, 3)[mask] - ref)) / np.max(np.abs(ref))
    assert err < 1e-10, err


def test_ensemble_field_mixed_vs_fp64():
    P = sqbem.TrajParams(a_over_R=0.3, n_theta=24, sphere_level=2)
    rng = np.random.default_rng(11)
    R = 1.0 / P.a_over_R
    n = 3
    y = np.zeros((n, 6))
    for k in range(n):
        b = rng.uniform(0, 0.6) * (R - 1.0)
        ph = rng.uniform(0, 2 * math.pi)
        e = rng.normal(size=3)
        y[k] = [b * math.cos(ph), b * math.sin(ph), 0.0, *(e / np.linalg.norm(e))]
    alpha = rng.uniform(-5, 5, n)
    u64, _ = sqbem.ensemble_field(y, alpha, P, 13, 13, 21, 7.0, precision=sqbem.FP64)
    umx, t = sqbem.ensemble_field(y, alpha, P, 13, 13, 21, 7.0, precision=sqbem.MIXED)
    ok = ~np.isnan(u64)
    assert np.array_equal(ok, ~np.isnan(umx))
    err = np.max(np.abs(umx[ok] - u64[ok])) / np.max(np.abs(u64[ok]))
    print("mixed field rel err", err)
    assert err < 2e-5, err


def test_ensemble_streams_do_not_change_results(monkeypatch):
    """100 swimmers = 3 groups of at most 48, solved concurrently on several
    streams: bitwise the single-stream trajectories and field"""
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.25, n_theta=8, sphere_level=1)
    rng = np.random.default_rng(31)
    y0 = _initial_states(P, 100, rng)
    alpha = rng.uniform(-4, 4, 100)
    out = {}
    for ns in ("1", "4"):
        monkeypatch.setenv("SQBEM_STREAMS", ns)
        s, U, Om, st, _ = sqbem.trajectory_ensemble(y0, alpha, P, 2, scheme=1, precision=sqbem.MIXED)
        u, _ = sqbem.ensemble_field(s[:, -1, :], alpha, P, 5, 5, 7, 4.0, precision=sqbem.MIXED)
        out[ns] = (s, U, u)
    for a, b in zip(out["1"], out["4"]):
        np.testing.assert_array_equal(a, b)
