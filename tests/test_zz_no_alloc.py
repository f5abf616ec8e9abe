"""sqbem_velocity_at_noalloc: the field evaluation for callers that cannot
allocate device memory (they hand in device buffers they own, e.g. from a
pre-reserved arena whose owner forbids allocations while it runs).  Checked
through the C ABI against sqbem_velocity_at, the allocating entry point, on
two calls in a row with different geometry and inputs, so the second call must
not see anything the first one left in the shared scratch array; and a call
that overflows the near-panel limit followed by a normal one.

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu


# Two geometries: the second has fewer panels and a different tube and sphere,
# so every panel record the second call reads must be its own, not one the
# first call left in the shared scratch array.
CASES = {1: dict(n_theta=12, L_over_R=4.0, level=2, beta=0.4),
         2: dict(n_theta=8, L_over_R=3.0, level=1, beta=0.2)}


def _case(seed):
    c = CASES[seed]
    rng = np.random.default_rng(seed)
    R = 10.0 / 3
    tube = sqbem.swimmer_tube_mesh(R, c["L_over_R"] * R, 1.0, c["n_theta"], 4)
    b = c["beta"] * (R - 1.0)
    sph = sqbem.icosphere(1.0, c["level"], (b, 0.0, 0.0))
    allm = sqbem.merge(tube, sph)
    u = rng.normal(size=(allm.P, 3))
    f = rng.normal(size=(allm.P, 3))
    n = 300
    pts = np.stack([rng.uniform(-0.8 * R, 0.8 * R, n), rng.uniform(-0.5 * R, 0.5 * R, n),
                    rng.uniform(-0.4 * c["L_over_R"] * R, 0.4 * c["L_over_R"] * R, n)], axis=1)
    keep = np.linalg.norm(pts - np.array([b, 0, 0]), axis=1) > 1.1
    return allm, u, f, pts[keep]


def _crowded_case():
    """300 small triangles within 0.02 of the origin, evaluated at the origin:
    every panel is near (distance < 3 h), more than the 256 near panels one
    point may have, so the call must fail cleanly"""
    rng = np.random.default_rng(7)
    V = []
    for _ in range(300):
        c = rng.normal(size=3)
        c *= rng.uniform(0.005, 0.02) / np.linalg.norm(c)
        V.append(np.concatenate([c, c + np.array([0.01, 0.0, 0.0]), c + np.array([0.0, 0.01, 0.0])]))
    allm = sqbem.Mesh(np.array(V), np.zeros(300, dtype=np.int32))
    u = rng.normal(size=(300, 3))
    f = rng.normal(size=(300, 3))
    return allm, u, f, np.zeros((1, 3))


def _noalloc(torch, allm, u, f, pts, precision):
    """one call through the C ABI with device buffers the caller owns; returns
    (status, output)"""
    dev = torch.device("cuda:0")
    V = torch.tensor(allm.V, dtype=torch.float64, device=dev).contiguous()
    du = torch.tensor(u, dtype=torch.float64, device=dev).contiguous()
    df = torch.tensor(f, dtype=torch.float64, device=dev).contiguous()
    dp = torch.tensor(pts, dtype=torch.float64, device=dev).contiguous()
    out = torch.full((pts.shape[0], 3), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = sqbem.lib().sqbem_velocity_at_noalloc(allm.P, V.data_ptr(), du.data_ptr(), df.data_ptr(), 1.0, pts.shape[0],
                                               dp.data_ptr(), out.data_ptr(), precision, ctypes.c_void_p(stream))
    return rc, out.cpu().numpy()


def _check_against_allocating(torch, seed, precision):
    allm, u, f, pts = _case(seed)
    ref = sqbem.velocity_at(allm, u, f, 1.0, pts, precision)
    rc, got = _noalloc(torch, allm, u, f, pts, precision)
    assert rc == sqbem.OK, sqbem.lib().sqbem_last_error().decode()
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale, seed


@pytest.mark.parametrize("precision", [sqbem.FP64, sqbem.MIXED])
def test_noalloc_matches_allocating_entry_point(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    for seed in (1, 2):  # two calls in a row, different geometry and inputs
        _check_against_allocating(torch, seed, precision)


def test_noalloc_overflow_then_normal_call():
    """a call that trips the near-panel limit fails with SQBEM_ERR_ARG; the
    next call (which must clear the overflow flag the first one set in the
    shared scratch) succeeds and matches the allocating entry point"""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    allm, u, f, pts = _crowded_case()
    rc, _ = _noalloc(torch, allm, u, f, pts, sqbem.FP64)
    assert rc == sqbem.ERR_ARG
    assert b"256 near panels" in sqbem.lib().sqbem_last_error()
    _check_against_allocating(torch, 2, sqbem.FP64)


def test_noalloc_rejects_too_many_panels():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda:0")
    P = 16385
    buf = torch.zeros(9 * P, dtype=torch.float64, device=dev)
    pts = torch.zeros(3, dtype=torch.float64, device=dev)
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    rc = sqbem.lib().sqbem_velocity_at_noalloc(P, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), 1.0, 1,
                                               pts.data_ptr(), out.data_ptr(), sqbem.FP64, None)
    assert rc == sqbem.ERR_ARG
    assert b"16384" in sqbem.lib().sqbem_last_error()
