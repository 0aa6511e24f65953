"""The adjoint (reverse-mode) engine: gradients of the mass-norm loss of u(T)
with respect to u0 and the diffusion field kappa, against the CPU reference
adjoint, central finite differences of the GPU forward, the dot-product
identity, checkpoint spacing and the torch.autograd bridge."""
from __future__ import annotations

import numpy as np
import pytest

import _adjoint_ref as ar
import ads_gb300 as ads
import oracle

pytestmark = pytest.mark.gpu


def _setup(p, elements, nsteps, dt, every=0, seed=0):
    import torch

    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    adj = ads.Adjoint(ctx, nsteps, dt, every)
    rng = np.random.default_rng(seed)
    n = ctx.size
    host = dict(u0=rng.uniform(-1, 1, n), kappa=1 + 0.5 * rng.uniform(-1, 1, n), target=rng.uniform(-1, 1, n))
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    return ctx, adj, host, dev


def _grads(ctx, adj, dev):
    import torch

    uT = torch.empty_like(dev["u0"])
    adj.forward(dev["u0"], dev["kappa"], uT)
    scratch, dL = torch.empty_like(uT), torch.empty_like(uT)
    loss = ads.mass_loss(ctx, uT, dev["target"], scratch, dL)
    gu, gk = torch.empty_like(uT), torch.empty_like(uT)
    adj.backward(dL, gu, gk)
    ctx.synchronize()
    return loss, gu.cpu().numpy(), gk.cpu().numpy(), uT


@pytest.mark.parametrize("p,elements,nsteps,dt", [((2, 2, 2), (5, 4, 6), 6, 1e-3), ((3, 3), (7, 6), 5, 1e-3),
                                                   ((4, 4, 4), (3, 3, 3), 3, 1e-4), ((1, 1, 1), (6, 5, 4), 5, 1e-3),
                                                   ((3, 3, 3), (4, 3, 5), 4, 1e-4), ((2, 2, 2), (9, 8, 7), 3, 1e-4)])
def test_adjoint_against_cpu_reference(p, elements, nsteps, dt, cuda):
    """3D backward steps run R(kappa) mu and the kappa gradient as one fused
    element pass (every degree 1-4 here); 2D runs the two kernels."""
    ctx, adj, h, dev = _setup(p, elements, nsteps, dt, seed=sum(elements))
    loss, gu, gk, _ = _grads(ctx, adj, dev)
    pr = oracle.Problem(list(p), list(elements))
    L, ru, rk = ar.gradients(pr, h["u0"], h["kappa"], dt, nsteps, h["target"])
    assert abs(loss - L) <= 1e-12 * abs(L)
    assert oracle.rel_l2(gu, ru) <= 1e-11
    assert oracle.rel_l2(gk, rk) <= 1e-11


def test_dot_product_identity(cuda):
    """<A x, y> = <x, A^T y> for the linear map u0 -> u(T) at fixed kappa."""
    import torch

    ctx, adj, h, dev = _setup((2, 2, 2), (8, 7, 6), 12, 5e-4, seed=3)
    rng = np.random.default_rng(33)
    x = torch.from_numpy(rng.standard_normal(ctx.size)).cuda()
    y = torch.from_numpy(rng.standard_normal(ctx.size)).cuda()
    Ax = torch.empty_like(x)
    adj.forward(x, dev["kappa"], Ax)
    ATy, gk = torch.empty_like(x), torch.empty_like(x)
    adj.backward(y, ATy, gk)
    ctx.synchronize()
    lhs, rhs = float(Ax @ y), float(x @ ATy)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


def test_finite_differences_of_the_gpu_forward(cuda):
    import torch

    ctx, adj, h, dev = _setup((2, 2, 2), (6, 6, 6), 20, 1e-4, seed=5)
    loss0, gu, gk, _ = _grads(ctx, adj, dev)
    scratch, dL, uT = (torch.empty_like(dev["u0"]) for _ in range(3))

    def loss(u0, kappa):
        adj.forward(u0, kappa, uT)
        return ads.mass_loss(ctx, uT, dev["target"], scratch, dL)

    for seed in range(4):
        d = torch.from_numpy(np.random.default_rng(200 + seed).standard_normal(ctx.size)).cuda()
        for which, g in (("u0", gu), ("kappa", gk)):
            hstep = 1e-6
            up = {k: v.clone() for k, v in dev.items()}
            dn = {k: v.clone() for k, v in dev.items()}
            up[which] += hstep * d
            dn[which] -= hstep * d
            fd = (loss(up["u0"], up["kappa"]) - loss(dn["u0"], dn["kappa"])) / (2 * hstep)
            an = float(np.dot(g, d.cpu().numpy()))
            assert abs(fd - an) <= 1e-6 * max(abs(fd), abs(an)), (which, fd, an)


def test_checkpoint_spacing_does_not_change_gradients(cuda):
    grads = []
    for every in (1, 3, 0, 17):
        ctx, adj, h, dev = _setup((2, 2), (9, 8), 17, 1e-3, every=every, seed=7)
        loss, gu, gk, _ = _grads(ctx, adj, dev)
        grads.append((gu, gk))
    for gu, gk in grads[1:]:
        np.testing.assert_array_equal(gu, grads[0][0])
        np.testing.assert_array_equal(gk, grads[0][1])


def test_torch_autograd_bridge(cuda):
    from ads_gb300.autograd import HeatRollout, MassNorm

    ctx, adj, h, dev = _setup((2, 2, 2), (5, 5, 5), 6, 1e-3, seed=9)
    loss_ref, gu_ref, gk_ref, _ = _grads(ctx, adj, dev)
    rollout = HeatRollout(ctx, 6, 1e-3)
    u0 = dev["u0"].clone().requires_grad_(True)
    kappa = dev["kappa"].clone().requires_grad_(True)
    loss = MassNorm.apply(rollout(u0, kappa), dev["target"], ctx)
    loss.backward()
    assert abs(float(loss.detach()) - loss_ref) <= 1e-14 * abs(loss_ref)
    np.testing.assert_array_equal(u0.grad.cpu().numpy(), gu_ref)
    np.testing.assert_array_equal(kappa.grad.cpu().numpy(), gk_ref)


def test_adjoint_outliving_its_context_fails_cleanly(cuda):
    """Destroying the context first detaches its adjoints: their calls then
    report an error and their destruction stays safe (as happens when a
    garbage collector finalises both in arbitrary order)."""
    import torch

    ctx, adj, _, dev = _setup((2, 2), (6, 5), 4, 1e-3)
    ctx.close()
    uT = torch.empty_like(dev["u0"])
    with pytest.raises(RuntimeError, match="context was destroyed"):
        adj.forward(dev["u0"], dev["kappa"], uT)
    adj.close()
