"""sqbem_velocity_at_noalloc: the field evaluation for callers that cannot
allocate device memory (they hand in device buffers they own, e.g. from a
pre-reserved arena).  Checked through the C ABI against sqbem_velocity_at, the
allocating entry point, on two calls in a row with different inputs, so the
second call must not see anything the first one left in the shared scratch.

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
pytestmark = pytest.mark.gpu


def _case(seed):
    rng = np.random.default_rng(seed)
    R = 10.0 / 3
    tube = sqbem.swimmer_tube_mesh(R, 4 * R, 1.0, 12, 4)
    b = 0.4 * (R - 1.0)
    sph = sqbem.icosphere(1.0, 2, (b, 0.0, 0.0))
    allm = sqbem.merge(tube, sph)
    u = rng.normal(size=(allm.P, 3))
    f = rng.normal(size=(allm.P, 3))
    n = 300
    pts = np.stack([rng.uniform(-0.8 * R, 0.8 * R, n), rng.uniform(-0.5 * R, 0.5 * R, n),
                    rng.uniform(-1.6 * R, 1.6 * R, n)], axis=1)
    keep = np.linalg.norm(pts - np.array([b, 0, 0]), axis=1) > 1.1
    return allm, u, f, pts[keep]


def _noalloc(torch, allm, u, f, pts, precision):
    dev = torch.device("cuda:0")
    V = torch.tensor(allm.V, dtype=torch.float64, device=dev).contiguous()
    du = torch.tensor(u, dtype=torch.float64, device=dev).contiguous()
    df = torch.tensor(f, dtype=torch.float64, device=dev).contiguous()
    dp = torch.tensor(pts, dtype=torch.float64, device=dev).contiguous()
    out = torch.full((pts.shape[0], 3), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = sqbem.lib().sqbem_velocity_at_noalloc(allm.P, V.data_ptr(), du.data_ptr(), df.data_ptr(), 1.0, pts.shape[0],
                                               dp.data_ptr(), out.data_ptr(), precision, ctypes.c_void_p(stream))
    assert rc == sqbem.OK, sqbem.lib().sqbem_last_error().decode()
    return out.cpu().numpy()


@pytest.mark.parametrize("precision", [sqbem.FP64, sqbem.MIXED])
def test_noalloc_matches_allocating_entry_point(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    for seed in (1, 2):  # two calls in a row, different inputs
        allm, u, f, pts = _case(seed)
        ref = sqbem.velocity_at(allm, u, f, 1.0, pts, precision)
        got = _noalloc(torch, allm, u, f, pts, precision)
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale, seed


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
