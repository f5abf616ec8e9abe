"""Failure paths of the device-side safeguards, made to happen without faulting
the GPU: one of the tensor-core GEMM's bounded mbarrier waits is pointed at a
barrier that nothing completes (sqbem_test_gemm_stall) with a short limit, so
it runs out (SQBEM_ERR_TIMEOUT, the library stays usable); and the
mixed-precision refinement is allowed no step (SQBEM_ERR_NOT_CONVERGED).  The
limits come from sqbem_set_limits and are restored after each test."""
import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu


@pytest.fixture
def limits():
    yield sqbem.set_limits
    sqbem.lib().sqbem_test_gemm_stall(0)
    sqbem.set_limits(-1, -1)


def _gemm_case(M=512, N=512, K=8192, seed=3):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    return A, B


def test_gemm_wait_expiry_reports_timeout_and_recovers(limits):
    A, B = _gemm_case()
    limits(2_000_000, -1)  # about 1 ms of SM clock per wait
    assert sqbem.lib().sqbem_test_gemm_stall(1) == sqbem.OK
    with pytest.raises(sqbem.BEMError) as ei:
        sqbem.gemm_mixed(A, B)
    assert ei.value.code == sqbem.ERR_TIMEOUT
    assert "bounded wait" in str(ei.value)
    limits(-1, -1)
    C = sqbem.gemm_mixed(A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    assert np.max(np.abs(C - ref)) < 1e-3 * np.max(np.abs(ref))


def test_refinement_cap_reports_not_converged(limits):
    a, lam, beta = 1.0, 0.3, 0.4
    R = a / lam
    b = beta * (R - a)
    e = np.array([0.0, 0.0, 1.0])
    tube = sqbem.Tube(R, 4 * R, a, 8, precision=sqbem.MIXED)
    s = sqbem.SwimmerSolver(tube, sqbem.icosphere(a, 1, (b, 0, 0)), (b, 0, 0), precision=sqbem.MIXED)
    slips = [s.slip(e, 1, 0), s.slip(e, 0, 1)]
    limits(-1, 0)
    with pytest.raises(sqbem.BEMError) as ei:
        s.solve_free(slips)
    assert ei.value.code == sqbem.ERR_NOT_CONVERGED
    inst = dict(a_over_R=lam, beta=beta, L_over_R=4.0, e=(0, 0, 1.0), n_theta=8, n_r=4, sphere_level=1)
    with pytest.raises(sqbem.BEMError) as ei:
        sqbem.kinematics_batch([inst], sqbem.MIXED)
    assert ei.value.code == sqbem.ERR_NOT_CONVERGED
    limits(-1, -1)
    m = s.solve_free(slips)
    it, res = s.refinement()
    assert 1 <= it and res <= 1e-8
    assert np.all(np.isfinite(m[0].U))


def test_set_limits_rejects_absurd_cap():
    with pytest.raises(sqbem.BEMError):
        sqbem.set_limits(-1, 5000)
