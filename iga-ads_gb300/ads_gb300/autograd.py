"""torch.autograd bridge for the adjoint of the kappa-weighted heat run.

    rollout = HeatRollout(ctx, nsteps=200, dt=1e-6)       # sqrt(N) checkpoints
    uT = rollout(u0, kappa)                                # torch CUDA float64
    loss = MassNorm.apply(uT, target, ctx)                 # (u-t)^T M (u-t)
    loss.backward()                                        # u0.grad, kappa.grad

Both Functions call the C-ABI (adsg_adjoint_*, adsg_mass_loss); no torch
arithmetic is involved in the forward or backward of the step itself.
"""
from __future__ import annotations

import torch

from . import Adjoint, Context, mass_loss


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(fctx, u0, kappa, adj):
        u0c, kc = u0.detach().contiguous(), kappa.detach().contiguous()
        uT = torch.empty_like(u0c)
        adj.forward(u0c, kc, uT)
        fctx.adj = adj
        return uT

    @staticmethod
    def backward(fctx, grad_uT):
        adj = fctx.adj
        g = grad_uT.detach().contiguous()
        gu = torch.empty_like(g)
        gk = torch.empty_like(g)
        adj.backward(g, gu, gk)
        adj.ctx.synchronize()
        return gu, gk, None


class HeatRollout:
    """nsteps of u <- M^{-1} R(kappa) u as a differentiable function of (u0, kappa)."""

    def __init__(self, ctx: Context, nsteps: int, dt: float, checkpoint_every: int = 0):
        self.adj = Adjoint(ctx, nsteps, dt, checkpoint_every)

    def __call__(self, u0, kappa):
        return _Rollout.apply(u0, kappa, self.adj)


class MassNorm(torch.autograd.Function):
    """L = (u - t)^T (Mx (x) My (x) Mz) (u - t)."""

    @staticmethod
    def forward(fctx, u, target, ctx):
        scratch = torch.empty_like(u)
        grad = torch.empty_like(u)
        val = mass_loss(ctx, u.detach().contiguous(), target.detach().contiguous(), scratch, grad)
        fctx.save_for_backward(grad)
        return torch.tensor(val, dtype=u.dtype, device=u.device)

    @staticmethod
    def backward(fctx, g):
        (grad,) = fctx.saved_tensors
        return grad * g, None, None
