"""The reference's acceptance checks, run on the GPU through this library.

The reference ships two test programs whose checks define "correct" for this
path: tests/test_duct_flow.cpp (7 checks) and tests/test_squirmer.cpp (18
checks in its default, quick mode: sphere level 2, n_theta = 24).  The same
physical checks are restated here with the same meshes, quantities and
tolerances (|value - target| <= tol), through the Python API over the C ABI,
in FP64.  Each test names the reference lines it restates.  The reference
programs themselves compile unchanged against the drop-in headers
(tests/test_dropin_compile.py)."""
import math

import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu

PI = math.pi
U0 = 2.0 / 3


def close(value, target, tol):
    assert abs(value - target) <= tol, (value, target, tol)


# ---------------------------------------------------------------- duct flow
@pytest.fixture(scope="module")
def duct():
    return sqbem.DuctFlow(1.0, 4.0, 24, 24, 6, 1.0)


def test_duct_flow_rate_and_linearity(duct):
    """test_duct_flow.cpp:27-38: Q / Q_exact at dP = 1 within 1e-2; Q / dP
    constant over dP in {0.5, 1, 2, 4} to 1e-10"""
    ratios = [duct.solve(dP, 0.0).Q / dP for dP in (0.5, 1.0, 2.0, 4.0)]
    close(duct.solve(1.0, 0.0).Q / duct.exact_Q(1.0), 1.0, 1e-2)
    close(max(abs(r / ratios[0] - 1) for r in ratios), 0.0, 1e-10)


def test_duct_interior_profile(duct):
    """test_duct_flow.cpp:40-56: u_z at mid-length along three azimuths within
    2e-2 of the parabola (relative to u_max), transverse velocity below 1e-3"""
    s = duct.solve(1.0, 0.0)
    pts = np.array([[0.95 * k / 19 * math.cos(a), 0.95 * k / 19 * math.sin(a), 2.0]
                    for a in (0.0, PI / 5, PI / 2) for k in range(20)])
    v = duct.velocity(s, pts)
    r = np.hypot(pts[:, 0], pts[:, 1])
    wmax = duct.exact_uz(0.0, 1.0)
    close(np.max(np.abs(v[:, 2] - duct.exact_uz(r, 1.0))) / wmax, 0.0, 2e-2)
    close(np.max(np.hypot(v[:, 0], v[:, 1])) / wmax, 0.0, 1e-3)


def test_duct_wall_traction(duct):
    """test_duct_flow.cpp:58-71: wall pressure linear in z (max error / dP
    below 1e-2) and mean wall shear -G R / 2 within 2e-2, away from the caps"""
    s = duct.solve(1.0, 0.0)
    m = duct.mesh
    G, L = 1.0 / 4.0, 4.0
    c = m.centroid
    keep = (m.tags == sqbem.WALL) & (c[:, 2] >= 0.5) & (c[:, 2] <= L - 0.5)
    er = c[keep].copy()
    er[:, 2] = 0.0
    er /= np.linalg.norm(er, axis=1)[:, None]
    f = s.f[keep]
    perr = np.max(np.abs(-np.sum(f * er, axis=1) - (1.0 - G * c[keep, 2])))
    close(np.mean(f[:, 2]) / (-G * 1.0 / 2), 1.0, 2e-2)
    close(perr, 0.0, 1e-2)


def test_duct_mesh_convergence():
    """test_duct_flow.cpp:73-84: the error in Q decreases under refinement"""
    errs = []
    for nth, nz, nr in ((12, 12, 3), (16, 16, 4), (20, 20, 5), (24, 24, 6)):
        d = sqbem.DuctFlow(1.0, 4.0, nth, nz, nr, 1.0)
        errs.append(abs(d.solve(1.0, 0.0).Q / d.exact_Q(1.0) - 1))
    assert all(errs[i] < errs[i - 1] for i in range(1, len(errs))), errs


# ---------------------------------------------------------------- squirmer (quick mode)
LEV, NTH = 2, 24
E = np.array([0.0, 0.0, 1.0])


def haberman_sayre(l):
    """towed sphere on the axis of a tube (Haberman & Sayre 1958), drag / 6 pi mu a U"""
    return (1 - 0.75857 * l ** 5) / (1 - 2.1050 * l + 2.0865 * l ** 3 - 1.7068 * l ** 5 + 0.72603 * l ** 6)


def blake(x, B1, B2):
    """Blake's (1971) squirmer flow in the lab frame, radius 1, swimming along +z"""
    r = np.linalg.norm(x)
    c = x[2] / r
    s = math.sqrt(max(0.0, 1 - c * c))
    ur = 2 / 3 * B1 * c / r ** 3 + (r ** -4 - r ** -2) * B2 * (3 * c * c - 1) / 2
    ut = 1 / 3 * B1 * s / r ** 3 + B2 * s * c / r ** 4
    rh = x / r
    eth = (c * rh - E) / max(s, 1e-12)
    return ur * rh + ut * eth


def towed_drag(s):
    return -s.force(s.solve_prescribed((0, 0, 1), (0, 0, 0)))[2] / (6 * PI)


def test_squirmer_unbounded():
    """test_squirmer.cpp:49-82 (quick): Stokes drag within 5e-3, swimming speed
    2 B1 / 3 within 6e-3, B2 mode motionless to 1e-10, Blake's field at
    r = 1.5 a within 2e-2 and at r = 3 a within 1e-2 (relative to U0)"""
    s = sqbem.SwimmerSolver(None, sqbem.icosphere(1.0, LEV), (0, 0, 0))
    close(towed_drag(s), 1.0, 5e-3)
    sl1, sl2 = s.slip(E, 1, 0), s.slip(E, 0, 1)
    m = s.solve_free([sl1, sl2])
    close(m[0].U[2] / U0, 1.0, 6e-3)
    close(np.linalg.norm(m[1].U) + np.linalg.norm(m[1].Om), 0.0, 1e-10)
    alpha = -3.0
    pts = np.array([[r * math.sin(PI * (i + 0.5) / 24), 0.0, r * math.cos(PI * (i + 0.5) / 24)]
                    for r in (1.1, 1.5, 3.0) for i in range(24)])
    v1, v2 = s.velocity(m[0], sl1, pts), s.velocity(m[1], sl2, pts)
    err = [np.linalg.norm(v1[k] + alpha * v2[k] - blake(pts[k], 1.0, alpha)) / U0 for k in range(len(pts))]
    close(max(err[24:48]), 0.0, 2e-2)  # r = 1.1 a is resolved on the fine mesh only (not checked in quick mode)
    close(max(err[48:72]), 0.0, 1e-2)


@pytest.fixture(scope="module")
def axis_runs():
    out = []
    for lam in (0.1, 0.2, 0.3, 0.4, 0.5, 0.6):
        t = sqbem.Tube(1 / lam, 4 / lam, 1.0, NTH)
        s = sqbem.SwimmerSolver(t, sqbem.icosphere(1.0, LEV), (0, 0, 0))
        K = towed_drag(s)
        m = s.solve_free([s.slip(E, 1, 0), s.slip(E, 0, 1)])
        out.append((lam, K, m))
    return out


def test_squirmer_on_axis(axis_runs):
    """test_squirmer.cpp:86-106: towed drag within 1e-2 of Haberman-Sayre for
    a/R <= 0.4 (four checks), swimming speed decreasing with a/R, B2 mode
    motionless on the axis to 1e-6"""
    prev, slower, b2 = U0, True, 0.0
    for lam, K, m in axis_runs:
        if lam <= 0.4 + 1e-9:
            close(K / haberman_sayre(lam), 1.0, 1e-2)
        slower &= m[0].U[2] < prev
        prev = m[0].U[2]
        b2 = max(b2, np.linalg.norm(m[1].U) + np.linalg.norm(m[1].Om))
    assert slower
    close(b2, 0.0, 1e-6)


def test_squirmer_reciprocal_theorem_and_decay():
    """test_squirmer.cpp:108-151: the Lorentz reciprocal theorem reproduces the
    swimming speed within 1e-2; the flow decays along the tube (max |u| / U0
    beyond |z| = 2 R below 2e-2) -- a/R = 0.3 on the axis"""
    R = 1 / 0.3
    t = sqbem.Tube(R, 4 * R, 1.0, NTH)
    s = sqbem.SwimmerSolver(t, sqbem.icosphere(1.0, LEV), (0, 0, 0))
    sl = s.slip(E, 1, 0)
    m = s.solve_free([sl])
    tow = s.solve_prescribed((0, 0, 1), (0, 0, 0))
    Fz = s.force(tow)[2]
    Urec = np.sum(np.sum(sl * tow.f_sphere, axis=1) * s.S.area) / Fz
    close(Urec / m[0].U[2], 1.0, 1e-2)
    nx, nz = 25, 57
    pts = np.array([[-0.97 * R + 1.94 * R * i / (nx - 1), 0.0, -2.2 * R + 4.4 * R * j / (nz - 1)]
                    for i in range(nx) for j in range(nz)])
    pts = pts[np.linalg.norm(pts, axis=1) >= 1.03]
    v = s.velocity(m[0], sl, pts)
    far = np.abs(pts[:, 2]) > 2 * R
    close(np.max(np.linalg.norm(v[far], axis=1)) / U0, 0.0, 2e-2)


def test_squirmer_off_axis():
    """test_squirmer.cpp:154-181 (quick, n_theta = 24): the B1 mode rotates away
    from the nearest wall and does not drift sideways (1e-8); the B2 > 0
    (puller) mode drifts away from the wall and does not rotate (1e-8); the
    axial speed decreases with the eccentricity"""
    R = 1 / 0.3
    t = sqbem.Tube(R, 4 * R, 1.0, NTH)
    rot_away, puller_away, uz_dec = True, True, True
    side_b1, rot_b2, prev = 0.0, 0.0, 1e9
    for beta in (0.0, 0.2, 0.4, 0.6, 0.75, 0.85):
        b = beta * (R - 1)
        s = sqbem.SwimmerSolver(t, sqbem.icosphere(1.0, LEV, (b, 0, 0)), (b, 0, 0))
        m = s.solve_free([s.slip(E, 1, 0), s.slip(E, 0, 1)])
        if beta > 0:
            rot_away &= m[0].Om[1] < 0
            puller_away &= m[1].U[0] < 0
        side_b1 = max(side_b1, abs(m[0].U[0]))
        rot_b2 = max(rot_b2, abs(m[1].Om[1]))
        uz_dec &= m[0].U[2] < prev + 1e-9
        prev = m[0].U[2]
    assert rot_away
    assert puller_away
    close(side_b1, 0.0, 1e-8)
    close(rot_b2, 0.0, 1e-8)
    assert uz_dec
