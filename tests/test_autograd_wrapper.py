"""The torch.autograd.Function around the adjoint, on the CPU: the library call
is replaced by an analytic stand-in with known Jacobians, so gradcheck tests the
wrapper's algebra (mode combination, alpha derivative, shapes) alone."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
sqbem = pytest.importorskip("sqbem")
import sqbem.autograd as sag  # noqa: E402

A = np.array([[[1.0, 0.2, -0.3], [0.0, 0.5, 0.1], [0.4, -0.2, 0.9]],
              [[-0.6, 0.1, 0.2], [0.3, 0.8, -0.5], [0.0, 0.2, 0.3]]])
B = np.array([[[0.2, 0.0, 0.1], [-0.3, 0.4, 0.0], [0.1, 0.1, -0.2]],
              [[0.5, -0.1, 0.0], [0.0, 0.2, 0.6], [-0.4, 0.3, 0.1]]])


def fake_evaluate(tube, center, e, level, a, mu):
    c = np.asarray(center, float)
    U = np.stack([A[m] @ np.sin(c) for m in range(2)])
    Om = np.stack([B[m] @ (c * c) for m in range(2)])
    dU = np.stack([A[m] * np.cos(c)[None, :] for m in range(2)])
    dOm = np.stack([B[m] * (2 * c)[None, :] for m in range(2)])
    return U, Om, dU, dOm


def test_gradcheck(monkeypatch):
    monkeypatch.setattr(sag, "_evaluate", fake_evaluate)
    c = torch.tensor([0.3, -0.7, 1.1], dtype=torch.float64, requires_grad=True)
    al = torch.tensor(-1.5, dtype=torch.float64, requires_grad=True)
    f = lambda cc, aa: sag.SwimmerKinematics.apply(cc, aa, None, (0.0, 0.0, 1.0), 2, 1.0, 1.0)
    assert torch.autograd.gradcheck(f, (c, al), eps=1e-6, atol=1e-8)


def test_forward_combines_modes(monkeypatch):
    monkeypatch.setattr(sag, "_evaluate", fake_evaluate)
    c = np.array([0.2, 0.4, -0.1])
    U, Om = sag.kinematics(None, c, 3.0)
    ref = fake_evaluate(None, c, None, 2, 1.0, 1.0)
    np.testing.assert_allclose(U.numpy(), ref[0][0] + 3.0 * ref[0][1])
    np.testing.assert_allclose(Om.numpy(), ref[1][0] + 3.0 * ref[1][1])
