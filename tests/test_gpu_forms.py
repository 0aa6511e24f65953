"""The general pointwise form (adsg_form_rhs) through the C-ABI against the
oracle's restatement of the reference's element loops:
heat_3d::compute_rhs (examples/heat/heat_3d.hpp:49-67),
scalability_3d::compute_rhs (examples/scalability/test3d.hpp:66-95, forcing
added without a test function) and flow::compute_rhs
(examples/flow/flow.hpp:77-98, nonlinear diffusion k exp(mi u) and a source)."""
from __future__ import annotations

import numpy as np
import pytest

import ads_gb300 as ads
import oracle

pytestmark = pytest.mark.gpu

CASES = [((2, 2, 2), (6, 5, 7)), ((4, 4, 4), (4, 5, 3)), ((3, 3), (12, 9)), ((2, 2), (20, 17)), ((1, 1, 1), (7, 6, 5))]


def _points(ctx):
    """Gauss-point coordinates (x, y[, z]) as x-fastest tensors over (rx, ry, rz)."""
    axes = [ctx.quad_points(d) for d in range(len(ctx.dims))]
    return [m.ravel() for m in np.meshgrid(*axes[::-1], indexing="ij")[::-1]]


def _setup(p, elements, seed):
    import torch

    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    pr = oracle.Problem(list(p), list(elements))
    u = np.random.default_rng(seed).uniform(-1, 1, pr.size)
    return ctx, pr, u, torch.from_numpy(u).cuda()


@pytest.mark.parametrize("p,elements", CASES)
def test_heat_form_equals_heat_rhs(p, elements, cuda):
    import torch

    ctx, pr, u, ud = _setup(p, elements, 1)
    dt = 1e-3
    r = torch.empty_like(ud)
    ctx.form_rhs(ud, r, alpha=1.0, beta=-dt)
    ref = pr.heat_rhs(u, dt)
    assert oracle.rel_l2(r.cpu().numpy(), ref) <= 1e-13
    h = torch.empty_like(ud)
    ctx.heat_rhs(ud, h, dt)
    assert oracle.rel_l2(r.cpu().numpy(), h.cpu().numpy()) <= 1e-13


@pytest.mark.parametrize("p,elements", CASES)
def test_scalability_forcing_form(p, elements, cuda):
    """test3d.hpp:57-63 forcing, added as dt f(x_q) w J to every dof of the element."""
    import torch

    ctx, pr, u, ud = _setup(p, elements, 2)
    dt = 1e-4
    X = _points(ctx)
    c = [x - 0.5 for x in X]
    r = np.sqrt(sum(ci * ci for ci in c))
    f = np.exp(-r) + 1 + np.prod([np.cos(np.pi * x) for x in X], axis=0)
    dq = torch.from_numpy(np.ascontiguousarray(dt * f)).cuda()
    out = torch.empty_like(ud)
    ctx.form_rhs(ud, out, alpha=1.0, beta=-dt, delta_q=dq)
    ref = pr.form_rhs(u, alpha=1.0, beta=-dt, delta_q=dt * f)
    assert oracle.rel_l2(out.cpu().numpy(), ref) <= 1e-13


@pytest.mark.parametrize("p,elements", CASES)
def test_flow_form(p, elements, cuda):
    """flow.hpp:77-98: (u v + dt(-k e^{mi u} grad u . grad v + h v)) w J with
    u(x_q) evaluated on the device; a smooth stand-in permeability and source."""
    import torch

    ctx, pr, u, ud = _setup(p, elements, 3)
    u *= 0.05
    ud *= 0.05
    dt, mi = 1e-3, 10.0
    uq = torch.empty(ctx.quad_size, dtype=torch.float64, device="cuda")
    ctx.eval_quad(ud, uq)
    X = _points(ctx)
    k = 1.0 + 0.5 * np.prod([np.sin(2 * np.pi * x) for x in X], axis=0)
    h = np.prod([x * (1 - x) for x in X], axis=0)
    beta = -dt * k * np.exp(mi * uq.cpu().numpy())
    gamma = dt * h
    out = torch.empty_like(ud)
    ctx.form_rhs(ud, out, alpha=1.0, beta_q=torch.from_numpy(beta).cuda(), gamma_q=torch.from_numpy(gamma).cuda())
    ref = pr.form_rhs(u, alpha=1.0, beta_q=beta, gamma_q=gamma)
    assert oracle.rel_l2(out.cpu().numpy(), ref) <= 1e-13


@pytest.mark.parametrize("p,elements", CASES[:3])
def test_pure_load_equals_load_vector(p, elements, cuda):
    """With no u terms the form is the load vector of compute_projection."""
    import torch

    ctx, pr, u, ud = _setup(p, elements, 4)
    X = _points(ctx)
    g = np.ascontiguousarray(np.prod([np.sin(np.pi * x) + 0.3 for x in X], axis=0))
    gd = torch.from_numpy(g).cuda()
    a, b = torch.empty_like(ud), torch.empty_like(ud)
    ctx.form_rhs(None, a, gamma_q=gd)
    ctx.load_vector(gd, b)
    ctx.synchronize()
    assert oracle.rel_l2(a.cpu().numpy(), b.cpu().numpy()) <= 1e-13
    assert oracle.rel_l2(a.cpu().numpy(), pr.form_rhs(None, gamma_q=g)) <= 1e-13


def test_form_argument_errors(cuda):
    import torch

    ctx, pr, u, ud = _setup((2, 2), (5, 5), 5)
    out = torch.empty_like(ud)
    with pytest.raises(RuntimeError, match="u is NULL"):
        ctx.form_rhs(None, out, alpha=1.0)
    mixed = ads.Context([ads.Dimension(2, 5), ads.Dimension(3, 5)])
    with pytest.raises(RuntimeError, match="same degree"):
        mixed.form_rhs(torch.zeros(mixed.size, dtype=torch.float64, device="cuda"),
                       torch.empty(mixed.size, dtype=torch.float64, device="cuda"), alpha=1.0)


@pytest.mark.parametrize("name", ["form_scalability_p2_e5", "form_scalability_p3_e4", "form_flow_p2_e6",
                                  "form_flow_p4_e3"])
def test_forms_against_reference_fixtures(name, cuda):
    """adsg_form_rhs against the reference's own scalability / flow loops
    (fixtures recorded from the compiled reference); flow's u at the Gauss
    points from adsg_eval_quad against the reference's eval_fun values."""
    import os

    import torch
    from conftest import GOLDEN
    from test_oracle_pin import form_fields

    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    p, E = int(g["p"]), int(g["elements"])
    ctx = ads.Context([ads.Dimension(p, E) for _ in range(3)])
    u = torch.from_numpy(g["u0"]).cuda()
    if "uq" in g:
        uq = torch.empty(ctx.quad_size, dtype=torch.float64, device="cuda")
        ctx.eval_quad(u, uq)
        assert oracle.rel_l2(uq.cpu().numpy(), g["uq"]) <= 1e-14
    f = form_fields(g)
    dev = {k: (torch.from_numpy(np.ascontiguousarray(v)).cuda() if isinstance(v, np.ndarray) else v)
           for k, v in f.items()}
    out = torch.empty_like(u)
    ctx.form_rhs(u, out, **dev)
    assert oracle.rel_l2(out.cpu().numpy(), g["rhs"]) <= 1e-13
