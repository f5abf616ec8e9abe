"""Batched kinematics (sqbem_kinematics_batch): the grouped mixed-precision
batch against the FP64 batch and against the reference fixtures."""
import numpy as np
import pytest

from conftest import golden

sqbem = pytest.importorskip("sqbem")
from sqbem import workloads  # noqa: E402

pytestmark = pytest.mark.gpu


def uo_err(a, b):
    """norm-wise relative error of (U_B1, Om_B1, U_B2, Om_B2) per instance"""
    return np.linalg.norm(a[:, :12] - b[:, :12], axis=1) / np.linalg.norm(b[:, :12], axis=1)


def rel(a, b):
    """max-abs relative error of a traction field"""
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(np.asarray(b))))


def test_batch_small_mixed_vs_fp64():
    rng = np.random.default_rng(5)
    insts = []
    for k in range(10):
        lam = rng.uniform(0.15, 0.55)
        e = rng.normal(size=3)
        e /= np.linalg.norm(e)
        insts.append(dict(a_over_R=lam, beta=rng.uniform(0, 0.8 * (1 - lam)), L_over_R=4.0, e=tuple(e),
                          n_theta=int(rng.choice([8, 12])), n_r=4, sphere_level=int(rng.choice([1, 2])),
                          towed=1))
    insts.append(dict(a_over_R=0.0, beta=0.0, L_over_R=4.0, e=(0, 0, 1.0), n_theta=0, n_r=4, sphere_level=2, towed=1))
    insts.append(dict(a_over_R=0.3, beta=0.0, L_over_R=4.0, e=(0, 0, 1.0), n_theta=12, n_r=4, sphere_level=1, towed=1))
    r64, t64 = sqbem.kinematics_batch(insts, sqbem.FP64)
    rmx, tmx = sqbem.kinematics_batch(insts, sqbem.MIXED)
    assert t64 > 0 and tmx > 0
    np.testing.assert_array_equal(r64[:, 13:15], rmx[:, 13:15])  # Nt, Ns
    assert np.all(uo_err(rmx, r64) < 1e-6), uo_err(rmx, r64)
    towed = ~np.isnan(r64[:, 12])
    assert towed.sum() == 2
    np.testing.assert_allclose(rmx[towed, 12], r64[towed, 12], rtol=1e-6)
    assert np.all(rmx[:, 15] >= 1)


def test_batch_fp64_matches_single_solves():
    g = golden("c2_l2")["l2_off"]
    inst = dict(a_over_R=g["a_over_R"], beta=g["beta"], L_over_R=4.0, e=tuple(g["e"]), n_theta=24, n_r=4,
                sphere_level=2, towed=0)
    r, _ = sqbem.kinematics_batch([inst], sqbem.FP64)
    ref = np.concatenate([g["B1"]["U"], g["B1"]["Om"], g["B2"]["U"], g["B2"]["Om"]])
    assert np.max(np.abs(r[0, :12] - ref)) < 1e-10 * np.max(np.abs(ref))


def test_batch_tractions_fp64_vs_reference():
    """sqbem_kinematics_batch_tractions: the f_sphere and f_tube of both slip
    modes (SwimmerSolution, swimmer.hpp:78-81) against the reference's dump"""
    g = golden("c2_l2")["l2_off"]
    inst = dict(a_over_R=g["a_over_R"], beta=g["beta"], L_over_R=4.0, e=tuple(g["e"]), n_theta=24, n_r=4,
                sphere_level=2, towed=0)
    r, _, fs, ft = sqbem.kinematics_batch([inst], sqbem.FP64, tractions=True)
    r0, _ = sqbem.kinematics_batch([inst], sqbem.FP64)
    np.testing.assert_array_equal(r[0, :12], r0[0, :12])
    for m, mode in enumerate(("B1", "B2")):
        assert rel(fs[0][m].reshape(-1), g[mode]["f_sphere"]) < 1e-10
        assert rel(ft[0][m].reshape(-1), g[mode]["f_tube"]) < 1e-10
    rm, _, fsm, ftm = sqbem.kinematics_batch([inst], sqbem.MIXED, tractions=True)
    for m, mode in enumerate(("B1", "B2")):
        assert rel(fsm[0][m].reshape(-1), g[mode]["f_sphere"]) < 1e-5
        assert rel(ftm[0][m].reshape(-1), g[mode]["f_tube"]) < 1e-5


@pytest.mark.slow
def test_batch_whole_sweep_mixed_vs_fp64():
    """every one of the 128 instances the headline benchmark times, as the
    squirmer B2/B1 = alpha each instance draws: U within 1e-6 of the FP64 path,
    Omega within 1e-6 in units of U/a (Omega vanishes on the axis), the stacked
    (U, Omega) of both slip modes within 1e-6; the sphere and wall tractions
    within 5e-5 max-abs relative (measured worst 1.3e-5, on the wall of a
    near-wall instance: the FP32 storage of the assembled blocks sets it)"""
    insts = workloads.sweep()
    rmx, _, fsm, ftm = sqbem.kinematics_batch(insts, sqbem.MIXED, tractions=True)
    r64, _, fs64, ft64 = sqbem.kinematics_batch(insts, sqbem.FP64, tractions=True)
    err = uo_err(rmx, r64)
    assert np.all(err < 1e-6), (float(err.max()), int(err.argmax()))
    for k, d in enumerate(insts):
        al = d["alpha"]
        U, U64 = rmx[k, 0:3] + al * rmx[k, 6:9], r64[k, 0:3] + al * r64[k, 6:9]
        W, W64 = rmx[k, 3:6] + al * rmx[k, 9:12], r64[k, 3:6] + al * r64[k, 9:12]
        assert np.linalg.norm(U - U64) < 1e-6 * np.linalg.norm(U64), k
        assert np.linalg.norm(W - W64) < 1e-6 * max(np.linalg.norm(W64), np.linalg.norm(U64)), k
        for A, B in ((fsm[k], fs64[k]), (ftm[k], ft64[k])):
            assert rel(A[0] + al * A[1], B[0] + al * B[1]) < 5e-5, k


def test_batch_sweep_instances_mixed_vs_fp64():
    """the first instances of the seeded sweep workload (n_theta = 24, levels 2 and 3)"""
    insts = workloads.sweep()[:6]
    r64, _ = sqbem.kinematics_batch(insts, sqbem.FP64)
    rmx, _ = sqbem.kinematics_batch(insts, sqbem.MIXED)
    err = uo_err(rmx, r64)
    assert np.all(err < 1e-6), err


def test_batch_rejects_bad_instances():
    with pytest.raises(sqbem.BEMError):
        sqbem.kinematics_batch([dict(a_over_R=1.5, beta=0.0, sphere_level=2)], sqbem.MIXED)
    with pytest.raises(sqbem.BEMError):
        sqbem.kinematics_batch([dict(a_over_R=0.3, beta=0.0, sphere_level=2, e=(0, 0, 2.0))], sqbem.MIXED)


def test_concurrent_chunks_match_sequential(monkeypatch):
    """groups run on several host threads / streams (SQBEM_STREAMS): the results
    are bitwise those of one stream (no shared scratch between the chunks)"""
    rng = np.random.default_rng(21)
    insts = []
    for k in range(10):
        insts.append(dict(a_over_R=float(rng.uniform(0.2, 0.5)), beta=float(rng.uniform(0, 0.4)), L_over_R=4.0,
                          e=(0.0, 0.0, 1.0), n_theta=int(rng.choice([10, 12, 14])), n_r=3,
                          sphere_level=int(rng.choice([1, 2])), towed=0))
    for prec in (sqbem.MIXED, sqbem.FP64):
        monkeypatch.setenv("SQBEM_STREAMS", "1")
        r1, _ = sqbem.kinematics_batch(insts, prec)
        monkeypatch.setenv("SQBEM_STREAMS", "3")
        for _ in range(2):
            r3, _ = sqbem.kinematics_batch(insts, prec)
            np.testing.assert_array_equal(r3[:, :12], r1[:, :12])
