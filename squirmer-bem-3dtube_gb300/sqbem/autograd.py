"""torch.autograd wrapper of the adjoint (sqbem_swimmer_adjoint).

``kinematics(tube, center, alpha, e)`` returns the free-swimming (U, Omega) of a
squirmer with B1 = 1, B2 = alpha and orientation e whose sphere (icosphere of
radius a at ``center``) sits in ``tube`` -- the solve_free of
src/swimmer.hpp:107-139 for the slip of src/utils/kernels.hpp:107-111 -- as a
differentiable function of ``center`` (3,) and ``alpha`` (scalar).  The forward
pass runs the FP64 GPU solve and the adjoint in one library call; the backward
pass only contracts the stored Jacobians with the incoming gradients:

  dU/dc     = dU_B1/dc + alpha dU_B2/dc   (adjoint, both slip modes at once)
  dU/dalpha = U_B2                         (U is linear in the slip)

Tensors are float64 on the host: the GPU work happens inside the library.
"""
import numpy as np
import torch

from . import FP64, SwimmerSolver, icosphere


def _evaluate(tube, center, e, level, a, mu):
    """U, Om (2, 3) and dU_dc, dOm_dc (2, 3, 3) for the slip modes (B1, B2)."""
    sphere = icosphere(a, level, center)
    s = SwimmerSolver(tube, sphere, center, mu, FP64)
    try:
        return s.adjoint([s.slip(e, 1.0, 0.0), s.slip(e, 0.0, 1.0)])
    finally:
        s.close()


class SwimmerKinematics(torch.autograd.Function):
    """(center, alpha) -> (U, Omega); backward by the stored adjoint Jacobians."""

    @staticmethod
    def forward(ctx, center, alpha, tube, e, level, a, mu):
        c = center.detach().to("cpu", torch.float64).numpy().copy()
        al = float(alpha.detach())
        U, Om, dU, dOm = _evaluate(tube, c, np.asarray(e, dtype=np.float64), level, a, mu)
        Jc = np.vstack([dU[0] + al * dU[1], dOm[0] + al * dOm[1]])  # (6, 3)
        Ja = np.concatenate([U[1], Om[1]])  # (6,)
        ctx.save_for_backward(torch.from_numpy(Jc), torch.from_numpy(Ja))
        ctx.alpha_shape = alpha.shape
        out_U = torch.from_numpy(U[0] + al * U[1]).to(center.dtype)
        out_Om = torch.from_numpy(Om[0] + al * Om[1]).to(center.dtype)
        return out_U, out_Om

    @staticmethod
    def backward(ctx, gU, gOm):
        Jc, Ja = ctx.saved_tensors
        g = torch.cat([gU.reshape(3), gOm.reshape(3)]).to(torch.float64)
        gc = (Jc.T @ g).to(gU.dtype)
        ga = (Ja @ g).reshape(ctx.alpha_shape).to(gU.dtype)
        return gc, ga, None, None, None, None, None


def kinematics(tube, center, alpha, e=(0.0, 0.0, 1.0), level=2, a=1.0, mu=1.0):
    """Differentiable (U, Omega) of a squirmer at ``center`` with B2/B1 = ``alpha``."""
    if not torch.is_tensor(center):
        center = torch.as_tensor(center, dtype=torch.float64)
    if not torch.is_tensor(alpha):
        alpha = torch.as_tensor(alpha, dtype=torch.float64)
    return SwimmerKinematics.apply(center, alpha, tube, tuple(float(x) for x in e), int(level), float(a), float(mu))
