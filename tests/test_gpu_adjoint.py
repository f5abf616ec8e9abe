"""Adjoint sensitivities on the GPU: d(U, Omega)/dc from the transpose solve and
the sphere-tube kernel derivatives, against central finite differences (step
1e-4, FP64) of the GPU solver and of the oracle, with detection of quadrature
rule changes between the two FD positions (kernels.hpp:74-75 picks the rule by
distance, so a step that moves a pair across d = 3, 1.5 or 0.75 makes a jump
that is not part of the derivative): where the nominal centre has such a
crossing, the comparison moves to the nearest rule-clean centre and the nominal
FD error is printed for the record."""
import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu

H = 1e-4
TOL = 1e-5  # max |adjoint - FD| relative to max |J|


def rules(targets, mesh):
    """quadrature level of every (target, panel) pair, kernels.hpp:74-75"""
    d = np.linalg.norm(mesh.centroid[None, :, :] - targets[:, None, :], axis=2) / mesh.h[None, :]
    return np.where(d < 0.75, 3, np.where(d < 1.5, 2, np.where(d < 3.0, 1, 0)))


def rule_change(tube_mesh, level, a, c, axis):
    """True if some sphere-tube pair changes rule between c - h e_axis and c + h e_axis"""
    out = []
    for sgn in (-1.0, 1.0):
        cc = np.array(c, float)
        cc[axis] += sgn * H
        S = sqbem.icosphere(a, level, cc)
        out.append((rules(tube_mesh.centroid, S), rules(S.centroid, tube_mesh)))
    return not (np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1]))


def clean_point(tube_mesh, level, c, axis, a=1.0):
    """c itself if the FD step along `axis` changes no quadrature rule there, else
    the first point of a fixed pseudo-random sequence of nearby centres (offsets
    of a few 1e-3) where it changes none; returns the point and whether it moved"""
    rng = np.random.default_rng(17 + axis)
    for k in range(400):
        cc = np.array(c, float) + (0.0 if k == 0 else rng.normal(size=3) * 2e-3 * (1 + k / 40))
        if not rule_change(tube_mesh, level, a, cc, axis):
            return cc, k > 0
    raise AssertionError("no rule-clean FD point near %s for axis %d" % (c, axis))


def check_fd(tube_mesh, level, c, solve, adjoint):
    """adjoint vs central FD, column by column, each at its rule-clean centre;
    returns (max |J_adj - J_fd| / max |J_fd|, number of moved columns)"""
    Ja = np.zeros((2, 6, 3))
    Jf = np.zeros((2, 6, 3))
    moved_n = 0
    for j in range(3):
        cj, moved = clean_point(tube_mesh, level, c, j)
        moved_n += moved
        Ja[:, :, j] = adjoint(cj)[:, :, j]
        cp, cm = cj.copy(), cj.copy()
        cp[j] += H
        cm[j] -= H
        Jf[:, :, j] = (solve(cp) - solve(cm)) / (2 * H)
    return np.max(np.abs(Ja - Jf)) / np.max(np.abs(Jf)), moved_n


def gpu_solve(tube, level, c, e, a=1.0):
    S = sqbem.icosphere(a, level, c)
    s = sqbem.SwimmerSolver(tube, S, c)
    k = s.solve_free([s.slip(e, 1, 0), s.slip(e, 0, 1)])
    s.close()
    return np.array([np.concatenate([k[m].U, k[m].Om]) for m in range(2)])  # (2, 6)


def adjoint_jacobian(tube, level, c, e, a=1.0):
    S = sqbem.icosphere(a, level, c)
    s = sqbem.SwimmerSolver(tube, S, c)
    U, Om, dU, dOm = s.adjoint([s.slip(e, 1, 0), s.slip(e, 0, 1)])
    s.close()
    return np.concatenate([U, Om], axis=1), np.concatenate([dU, dOm], axis=1)  # (2, 6), (2, 6, 3)


def test_adjoint_matches_gpu_fd_small():
    lam, beta = 0.3, 0.4
    R = 1.0 / lam
    tube = sqbem.Tube(R, 4 * R, 1.0, 12)
    c = np.array([beta * (R - 1.0), 0.13, 0.21])
    e = np.array([0.3, -0.2, 0.9])
    e /= np.linalg.norm(e)
    out, _ = adjoint_jacobian(tube, 1, c, e)
    np.testing.assert_allclose(out, gpu_solve(tube, 1, c, e), rtol=0, atol=1e-13)
    err, moved = check_fd(tube.mesh, 1, c, lambda x: gpu_solve(tube, 1, x, e),
                          lambda x: adjoint_jacobian(tube, 1, x, e)[1])
    print("moved", moved, "rel err", err)
    assert err < TOL, err


def test_adjoint_matches_oracle_fd(oracle):
    """against central differences of the oracle (the reference's FP64 algorithm)"""
    lam, beta = 0.35, 0.3
    R = 1.0 / lam
    tube = sqbem.Tube(R, 4 * R, 1.0, 8)
    otube = oracle.Tube(R, 4 * R, 1.0, 8)
    c = np.array([beta * (R - 1.0), -0.1, 0.05])
    e = np.array([0.0, 0.6, 0.8])

    def osolve(cc):
        S = oracle.icosphere(1.0, 1, cc)
        s = oracle.SwimmerSolver(otube, S, cc)
        k = s.solve_free([s.slip(e, 1, 0), s.slip(e, 0, 1)])
        return np.array([np.concatenate([k[m].U, k[m].Om]) for m in range(2)])

    out, _ = adjoint_jacobian(tube, 1, c, e)
    np.testing.assert_allclose(out, osolve(c), rtol=0, atol=1e-10 * np.max(np.abs(out)))
    err, moved = check_fd(tube.mesh, 1, c, osolve, lambda x: adjoint_jacobian(tube, 1, x, e)[1])
    print("moved", moved, "rel err", err)
    assert err < TOL, err


def test_adjoint_batch_config_instances():
    """the 32-instance adjoint workload (a/R ~ U[0.2, 0.5], beta ~ U[0, 0.5],
    level 2, n_theta = 24): batch output = single-instance adjoint at the nominal
    centre; adjoint vs central FD column by column at the nominal centre where the
    FD step changes no quadrature rule, else at the nearest rule-clean centre"""
    from sqbem import workloads
    inst = workloads.adjoint()
    res, secs = sqbem.adjoint_batch(inst)
    assert secs > 0
    worst, moved_n = 0.0, 0
    for k, d in enumerate(inst):
        R = 1.0 / d["a_over_R"]
        tube = sqbem.Tube(R, d["L_over_R"] * R, 1.0, d["n_theta"], d["n_r"])
        c = np.array([d["beta"] * (R - 1.0), 0.0, 0.0])
        e = np.array(d["e"])
        out, Jn = adjoint_jacobian(tube, 2, c, e)
        np.testing.assert_array_equal(np.concatenate([res["U"][k], res["Om"][k]], axis=1), out)
        np.testing.assert_array_equal(np.concatenate([res["dU_dc"][k], res["dOm_dc"][k]], axis=1), Jn)
        np.testing.assert_allclose(out, gpu_solve(tube, 2, c, e), rtol=0, atol=1e-12)
        err, moved = check_fd(tube.mesh, 2, c, lambda x: gpu_solve(tube, 2, x, e),
                              lambda x: adjoint_jacobian(tube, 2, x, e)[1])
        worst = max(worst, err)
        moved_n += moved
        print("instance", k, "moved columns", moved, "rel err", err)
        assert err < TOL, (k, err)
        tube.close()
    print("32 instances: worst rel err %.3e, %d of 96 columns moved to a rule-clean centre" % (worst, moved_n))


def test_B2_derivative_is_linear_mode():
    """d(U, Om)/d(B2/B1) = the B2-mode solution: U(alpha) = U_B1 + alpha U_B2"""
    R = 1.0 / 0.3
    tube = sqbem.Tube(R, 4 * R, 1.0, 12)
    c = np.array([0.5, 0.0, 0.0])
    e = np.array([0.0, 0.0, 1.0])
    out, _ = adjoint_jacobian(tube, 1, c, e)
    S = sqbem.icosphere(1.0, 1, c)
    s = sqbem.SwimmerSolver(tube, S, c)
    for alpha in (-3.0, 3.0):
        k = s.solve_free([s.slip(e, 1.0, alpha)])[0]
        np.testing.assert_allclose(np.concatenate([k.U, k.Om]), out[0] + alpha * out[1], rtol=0, atol=1e-12)


def test_unbounded_is_translation_invariant():
    c = np.array([0.3, -0.2, 0.1])
    S = sqbem.icosphere(1.0, 1, c)
    s = sqbem.SwimmerSolver(None, S, c)
    U, Om, dU, dOm = s.adjoint([s.slip((0, 0, 1), 1, 0)])
    assert np.all(dU == 0) and np.all(dOm == 0)
    assert abs(U[0, 2] - 2.0 / 3.0) < 0.02  # free-space squirmer speed 2 B1 / 3


def test_mixed_swimmer_rejected():
    R = 1.0 / 0.3
    tube = sqbem.Tube(R, 4 * R, 1.0, 8, precision=sqbem.MIXED)
    c = np.zeros(3)
    S = sqbem.icosphere(1.0, 1, c)
    s = sqbem.SwimmerSolver(tube, S, c, precision=sqbem.MIXED)
    with pytest.raises(sqbem.BEMError) as ei:
        s.adjoint([s.slip((0, 0, 1), 1, 0)])
    assert ei.value.code == sqbem.ERR_ARG


def test_autograd_function_backward():
    torch = pytest.importorskip("torch")
    from sqbem.autograd import kinematics
    R = 1.0 / 0.3
    tube = sqbem.Tube(R, 4 * R, 1.0, 12)
    rng = np.random.default_rng(5)
    for k in range(400):  # a centre whose FD steps change no rule on any axis
        c0 = np.array([0.6, 0.1, -0.2]) + (0.0 if k == 0 else rng.normal(size=3) * 2e-3 * (1 + k / 40))
        if not any(rule_change(tube.mesh, 1, 1.0, c0, j) for j in range(3)):
            break
    else:
        raise AssertionError("no rule-clean centre")
    c = torch.tensor(c0, dtype=torch.float64, requires_grad=True)
    alpha = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
    e = (0.0, 0.0, 1.0)
    U, Om = kinematics(tube, c, alpha, e, level=1)
    w = torch.tensor([0.3, -1.0, 2.0], dtype=torch.float64)
    v = torch.tensor([1.0, 0.5, -0.7], dtype=torch.float64)
    (U @ w + Om @ v).backward()

    def J(cc, al):
        u, o = kinematics(tube, torch.tensor(cc, dtype=torch.float64), torch.tensor(al, dtype=torch.float64), e,
                          level=1)
        return float(u @ w + o @ v)

    g = np.zeros(3)
    for j in range(3):
        cp, cm = c0.copy(), c0.copy()
        cp[j] += H
        cm[j] -= H
        g[j] = (J(cp, 2.0) - J(cm, 2.0)) / (2 * H)
    assert np.max(np.abs(c.grad.numpy() - g)) < TOL * np.max(np.abs(g))
    ga = (J(c0, 2.0 + H) - J(c0, 2.0 - H)) / (2 * H)  # exact up to rounding: U is linear in alpha
    assert abs(float(alpha.grad) - ga) < 1e-8 * max(1.0, abs(ga))
