"""Dirichlet steps through the C-ABI against the reference's own examples
(fixtures made by tests/golden/make_golden.py from those classes):

- examples/validation/validation.hpp: Dirichlet rows on all four sides of a
  2D grid, from the projection of sin(pi x) sin(pi y); after the run, the
  state, and its errorL2 / errorH1 against the exact solution
  e^{-2 pi^2 t} sin(pi x) sin(pi y) in percent of that solution's norms
  (validation.hpp:121-129), which doubles as a physics check;
- examples/heat/heat_2d.hpp: x.fix_left() and row x = 0 of every right-hand
  side set to the load vector of sin(pi y) (heat_2d.hpp:40-52), on the 2D
  p = 2, 32^2-element grid at dt = 1e-5 for 100 steps."""
from __future__ import annotations

import os

import numpy as np
import pytest

import ads_gb300 as ads
import oracle
from _tol import RUN, STEP, check
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _points(ctx, fun):
    axes = [ctx.quad_points(d) for d in range(len(ctx.dims))]
    mesh = np.meshgrid(*axes[::-1], indexing="ij")[::-1]
    val, grad = fun(*mesh)
    return np.ascontiguousarray(val.ravel()), np.ascontiguousarray(np.stack([g.ravel() for g in grad]).ravel())


def _exact(t):
    k = 2 * np.pi ** 2

    def f(x, y):
        sc = np.exp(-k * t)
        return (sc * np.sin(np.pi * x) * np.sin(np.pi * y),
                [sc * np.pi * np.cos(np.pi * x) * np.sin(np.pi * y), sc * np.pi * np.sin(np.pi * x) * np.cos(np.pi * y)])

    return f


def test_validation_problem_against_reference_and_exact_solution(cuda):
    import torch

    g = np.load(os.path.join(GOLDEN, "validation_2d_p2_e16.npz"))
    p, E, dt, N = int(g["p"]), int(g["elements"]), float(g["dt"]), int(g["nsteps"])
    n = E + p
    dims = [ads.Dimension(p, E) for _ in range(2)]
    for d in dims:
        d.fix_left()
        d.fix_right()
    ctx = ads.Context(dims)
    planes = [(0, 0, None), (0, n - 1, None), (1, 0, None), (1, n - 1, None)]
    # before(): projection of the initial state, boundary rows zeroed, solve
    f0, _ = _points(ctx, _exact(0.0))
    a = torch.empty(ctx.size, dtype=torch.float64, device=cuda)
    ctx.load_vector(torch.from_numpy(f0).to(cuda), a)
    ctx.set_planes(a, planes)
    ctx.ads_solve(a)
    b = torch.empty_like(a)
    for _ in range(N):
        ctx.heat_step_dirichlet(a, b, dt, planes)
        a, b = b, a
    ctx.synchronize()
    u = a.cpu().numpy()
    check(f"validation {n}x{n} p={p} {N} steps vs reference", oracle.rel_l2(u, g["uN"]), RUN)
    fT, gT = _points(ctx, _exact(N * dt))
    el2, eh1 = ctx.errors(a, torch.from_numpy(fT).to(cuda), torch.from_numpy(gT).to(cuda))
    nl2, nh1 = ctx.errors(torch.zeros_like(a), torch.from_numpy(fT).to(cuda), torch.from_numpy(gT).to(cuda))
    pl2, ph1 = 100 * el2 / nl2, 100 * eh1 / nh1
    print(f"[parity] validation errors vs exact solution: L2 {pl2:.6f}% H1 {ph1:.6f}% "
          f"(reference {float(g['errorL2_percent']):.6f}% {float(g['errorH1_percent']):.6f}%)")
    assert abs(pl2 - float(g["errorL2_percent"])) <= 1e-8 * float(g["errorL2_percent"])
    assert abs(ph1 - float(g["errorH1_percent"])) <= 1e-8 * float(g["errorH1_percent"])
    assert pl2 < 0.2 and ph1 < 0.5  # close to the exact solution
    # the Dirichlet rows stayed at zero
    U = u.reshape(n, n)
    assert np.all(U[0, :] == 0) and np.all(U[-1, :] == 0) and np.all(U[:, 0] == 0) and np.all(U[:, -1] == 0)


def test_heat_2d_dirichlet_row_against_reference(cuda):
    import torch

    g = np.load(os.path.join(GOLDEN, "heat2d_dirichlet_p2_e32.npz"))
    p, E, dt, N = int(g["p"]), int(g["elements"]), float(g["dt"]), int(g["nsteps"])
    x, y = ads.Dimension(p, E), ads.Dimension(p, E)
    x.fix_left()
    ctx = ads.Context([x, y])
    row = torch.from_numpy(np.ascontiguousarray(g["row"])).to(cuda)
    planes = [(0, 0, row)]
    # before(): the projection of init_state = 0, then heat_2d's solve
    a = torch.zeros(ctx.size, dtype=torch.float64, device=cuda)
    ctx.set_planes(a, planes)
    ctx.ads_solve(a)
    b = torch.empty_like(a)
    ctx.heat_step_dirichlet(a, b, dt, planes)
    ctx.synchronize()
    check("heat_2d Dirichlet 1 step vs reference", oracle.rel_l2(b.cpu().numpy(), g["u1"]), STEP)
    a, b = b, a
    for _ in range(N - 1):
        ctx.heat_step_dirichlet(a, b, dt, planes)
        a, b = b, a
    ctx.synchronize()
    check(f"heat_2d Dirichlet {N} steps vs reference", oracle.rel_l2(a.cpu().numpy(), g["uN"]), RUN)


def test_plane_arguments_are_checked(cuda):
    import torch

    ctx = ads.Context([ads.Dimension(2, 8), ads.Dimension(2, 6)])
    u = torch.zeros(ctx.size, dtype=torch.float64, device=cuda)
    with pytest.raises(ads.AdsError):
        ctx.set_planes(u, [(2, 0, None)])
    with pytest.raises(ads.AdsError):
        ctx.set_planes(u, [(1, 8, None)])
    v = torch.arange(ctx.size, dtype=torch.float64, device=cuda)
    vals = torch.full((10,), 7.0, dtype=torch.float64, device=cuda)
    ctx.set_planes(v, [(1, 3, vals), (0, 9, None)])
    ctx.synchronize()
    V = v.cpu().numpy().reshape(8, 10)
    ref = np.arange(80.0).reshape(8, 10)
    ref[3, :] = 7.0
    ref[:, 9] = 0.0
    np.testing.assert_array_equal(V, ref)
