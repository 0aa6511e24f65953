"""Gauss-point utilities through the C-ABI: the L2 projection (load vector of
reference include/ads/projection.hpp and projection + ads_solve), spline
evaluation at the Gauss points, normL2 / normH1 and errorL2 / errorH1
(reference include/ads/simulation/basic_simulation_3d.hpp:281-397), the last
pinned to the reference's own loops through tests/golden/norms_*.npz."""
from __future__ import annotations

import glob
import itertools
import os

import numpy as np
import pytest

import ads_gb300 as ads
import oracle
from _tol import mass_condition
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _grid_values(ctx, fun):
    """f at every Gauss point, x-fastest over (rx, ry, rz), and its gradient."""
    axes = [ctx.quad_points(d) for d in range(len(ctx.dims))]
    mesh = np.meshgrid(*axes[::-1], indexing="ij")[::-1]
    val, grad = fun(*mesh)
    return np.ascontiguousarray(val.ravel()), np.ascontiguousarray(np.stack([g.ravel() for g in grad]).ravel())


def _sin(*x):
    s = [np.sin(np.pi * xi) for xi in x]
    c = [np.pi * np.cos(np.pi * xi) for xi in x]
    val = np.prod(s, axis=0)
    grad = [np.prod([c[k] if k == d else s[k] for k in range(len(x))], axis=0) for d in range(len(x))]
    return val, grad


@pytest.mark.parametrize("nd,p,E", [(2, 2, 9), (3, 2, 6), (3, 4, 5), (2, 3, 11), (1, 2, 17)])
def test_projection_matches_reference_projection(nd, p, E, cuda):
    import torch

    dims = [ads.Dimension(p, E) for _ in range(nd)]
    ctx = ads.Context(dims)
    fq, _ = _grid_values(ctx, _sin)
    assert fq.size == ctx.quad_size
    f = torch.from_numpy(fq).cuda()
    b = torch.empty(ctx.size, dtype=torch.float64, device="cuda")
    ctx.load_vector(f, b)
    u = torch.empty_like(b)
    ctx.projection(f, u)
    ctx.synchronize()
    if nd >= 2:
        pr = oracle.Problem([p] * nd, [E] * nd)
        ref_b = pr.projection_sin()  # bit-identical to the reference's compute_projection
        assert oracle.rel_l2(b.cpu().numpy(), ref_b) <= 1e-14
        # the solve amplifies the load vector's rounding by up to cond(Mx (x) My (x) Mz)
        cond = np.prod([mass_condition(d.form_band(0).ravel(), p) for d in dims])
        assert oracle.rel_l2(u.cpu().numpy(), pr.ads_solve(ref_b)) <= max(1e-13, 1e-14 * cond)


@pytest.mark.parametrize("nd,p,E", [(2, 2, 7), (3, 3, 5), (3, 2, 8)])
def test_norms_match_oracle_quadratic_forms(nd, p, E, cuda):
    import torch

    dims = [ads.Dimension(p, E) for _ in range(nd)]
    ctx = ads.Context(dims)
    pr = oracle.Problem([p] * nd, [E] * nd)
    u = np.random.default_rng(E).uniform(-1, 1, ctx.size)
    l2, h1 = ctx.norms(torch.from_numpy(u).cuda())
    assert abs(l2 - np.sqrt(u @ pr.heat_rhs(u, 0.0))) <= 1e-13 * l2
    assert abs(h1 - np.sqrt(u @ pr.heat_rhs(u, -1.0))) <= 1e-13 * h1


def _eval_numpy(dims, u):
    """u and grad u at the Gauss points by direct quadrature loops (oracle-style)."""
    nd = len(dims)
    tabs = [d.tables() for d in dims]
    Q = [d.elements * d.quad_order for d in dims]
    n = [d.dofs() for d in dims]
    U = u.reshape(n[::-1])
    val = np.zeros(Q[::-1])
    grad = np.zeros([nd] + Q[::-1])
    for r in itertools.product(*[range(q) for q in Q]):
        vals = []
        for d in range(nd):
            e, k = divmod(r[d], dims[d].quad_order)
            P = dims[d].p
            row = tabs[d]["btab"].reshape(dims[d].elements, dims[d].quad_order, 2, P + 1)[e, k]
            vals.append((tabs[d]["first_dofs"][e], row))
        v = 0.0
        g = np.zeros(nd)
        for a in itertools.product(*[range(dims[d].p + 1) for d in range(nd)]):
            idx = tuple(vals[d][0] + a[d] for d in range(nd))[::-1]
            c = U[idx]
            b = [vals[d][1][0][a[d]] for d in range(nd)]
            db = [vals[d][1][1][a[d]] for d in range(nd)]
            v += c * np.prod(b)
            for d in range(nd):
                g[d] += c * np.prod([db[k] if k == d else b[k] for k in range(nd)])
        val[r[::-1]] = v
        grad[(slice(None),) + r[::-1]] = g
    return val.ravel(), grad.reshape(nd, -1)


@pytest.mark.parametrize("nd,p,E", [(2, 2, 5), (3, 2, 3), (2, 4, 4)])
def test_eval_quad_and_errors(nd, p, E, cuda):
    import torch

    dims = [ads.Dimension(p, E) for _ in range(nd)]
    ctx = ads.Context(dims)
    u = np.random.default_rng(p + E).uniform(-1, 1, ctx.size)
    ud = torch.from_numpy(u).cuda()
    val = torch.empty(ctx.quad_size, dtype=torch.float64, device="cuda")
    grad = torch.empty(nd * ctx.quad_size, dtype=torch.float64, device="cuda")
    ctx.eval_quad(ud, val, grad)
    ctx.synchronize()
    rv, rg = _eval_numpy(dims, u)
    assert oracle.rel_l2(val.cpu().numpy(), rv) <= 1e-14
    assert oracle.rel_l2(grad.cpu().numpy(), rg.ravel()) <= 1e-14
    fq, fg = _grid_values(ctx, _sin)
    l2, h1 = ctx.errors(ud, torch.from_numpy(fq).cuda(), torch.from_numpy(fg).cuda())
    axes = [ctx.quad_points(d) for d in range(nd)]
    W1 = []
    for d in range(nd):
        t = dims[d].tables()
        W1.append(np.repeat(t["J"], dims[d].quad_order) * np.tile(t["w"], dims[d].elements))
    W = W1[0]
    for w in W1[1:]:
        W = np.multiply.outer(w, W)
    W = W.ravel()
    ref_l2 = np.sqrt(np.sum(W * (rv - fq) ** 2))
    ref_h1 = np.sqrt(ref_l2 ** 2 + np.sum(W * ((rg - fg.reshape(nd, -1)) ** 2).sum(axis=0)))
    assert abs(l2 - ref_l2) <= 1e-13 * ref_l2
    assert abs(h1 - ref_h1) <= 1e-13 * ref_h1
    l2b, h1b = ctx.errors(ud, torch.from_numpy(fq).cuda())
    assert h1b is None and abs(l2b - l2) <= 1e-15 * l2


def test_projection_converges_to_the_function(cuda):
    """The projected sin field approaches sin: L2 error falls like h^(p+1)."""
    import torch

    errs = []
    for E in (8, 16, 32):
        dims = [ads.Dimension(2, E) for _ in range(2)]
        ctx = ads.Context(dims)
        fq, fg = _grid_values(ctx, _sin)
        f = torch.from_numpy(fq).cuda()
        u = torch.empty(ctx.size, dtype=torch.float64, device="cuda")
        ctx.projection(f, u)
        errs.append(ctx.errors(u, f)[0])
    rates = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(2.7 < r < 3.3 for r in rates), rates


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "norms_*.npz"))), ids=os.path.basename)
def test_norms_and_errors_match_the_reference_loops(path, cuda):
    """adsg_norms / adsg_errors against the reference's own normL2, normH1,
    errorL2 and errorH1 (basic_simulation_2d/3d.hpp quadrature loops, run by
    tests/golden/make_golden.py) on a seeded spline and prod sin(pi x_d)."""
    import torch

    g = np.load(path)
    nd, p, E = int(g["ndim"]), int(g["p"]), int(g["elements"])
    dims = [ads.Dimension(p, E) for _ in range(nd)]
    ctx = ads.Context(dims)
    u = torch.from_numpy(np.ascontiguousarray(g["u"])).cuda()
    l2, h1 = ctx.norms(u)
    fq, fg = _grid_values(ctx, _sin)
    el2, eh1 = ctx.errors(u, torch.from_numpy(fq).cuda(), torch.from_numpy(fg).cuda())
    nl2, nh1 = ctx.errors(torch.zeros_like(u), torch.from_numpy(fq).cuda(), torch.from_numpy(fg).cuda())
    for name, got, ref in (("normL2", l2, g["normL2"]), ("normH1", h1, g["normH1"]), ("errorL2", el2, g["errorL2"]),
                           ("errorH1", eh1, g["errorH1"]), ("f normL2", nl2, g["f_normL2"]),
                           ("f normH1", nh1, g["f_normH1"])):
        rel = abs(got - float(ref)) / float(ref)
        print(f"[parity] {os.path.basename(path)} {name}: {got:.15e} vs reference {float(ref):.15e} (rel {rel:.1e})")
        assert rel <= 1e-13, (name, got, float(ref))
