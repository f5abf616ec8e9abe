"""The tube's rotational symmetry used by the mixed assembly (CPU): for the tube
of every sweep instance (and a few other meshes) the library finds n_theta
sectors, and every panel's vertices are its representative's vertices rotated by
its sector angle, in the same order."""
import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
from sqbem import workloads  # noqa: E402


def _check(R, L, a, nth, nr):
    nb, sector, rep = sqbem.tube_symmetry(R, L, a, nth, nr)
    m = sqbem.swimmer_tube_mesh(R, L, a, nth, nr)
    assert nb * nth == m.P
    reps = np.flatnonzero(sector == 0)
    assert len(reps) == nb and np.array_equal(rep[reps], np.arange(nb))
    # each (representative, sector) pair names exactly one panel
    assert len(set(zip(rep.tolist(), sector.tolist()))) == m.P
    ang = 2 * np.pi * sector / nth
    c, s = np.cos(ang), np.sin(ang)
    V = m.V.reshape(-1, 3, 3)
    W = V[reps[rep]]  # representative vertices, rotated by the panel's sector
    rot = np.stack([c[:, None] * W[:, :, 0] - s[:, None] * W[:, :, 1],
                    s[:, None] * W[:, :, 0] + c[:, None] * W[:, :, 1], W[:, :, 2]], axis=2)
    assert np.max(np.abs(rot - V)) <= 1e-12 * np.max(np.abs(V))


def test_sweep_tubes_are_symmetric():
    seen = set()
    for d in workloads.sweep():
        key = (d["a_over_R"], d["n_theta"], d["n_r"], d["L_over_R"])
        if key in seen:
            continue
        seen.add(key)
        R = 1.0 / d["a_over_R"]
        _check(R, d["L_over_R"] * R, 1.0, d["n_theta"], d["n_r"])
    assert len(seen) >= 100


@pytest.mark.parametrize("nth,nr", [(10, 2), (24, 4), (36, 4), (7, 3)])
def test_other_tubes_are_symmetric(nth, nr):
    _check(10.0 / 3, 40.0 / 3, 1.0, nth, nr)
