"""The largest tensor a context accepts: 1290^3 = 2 146 689 000 dofs, just
under the 2^31 limit (17.2 GB per tensor, ~120 GB of device memory with the
context's work tensors).  Index arithmetic near the end of such a tensor is
where 32-bit overflow would show, so the checks reach it directly:

- the heat RHS at sampled points, the last one among them, against the same
  sum formed on the host from the 5x5x5 neighbourhood of the input and the
  oracle's 1D mass and stiffness bands (M_x (x) M_y (x) M_z - dt (K_x M_y M_z
  + M_x K_y M_z + M_x M_y K_z)) u, at 1e-13 of the terms' magnitude;
- the solve inverts the mass apply (the RHS at dt = 0) over the whole tensor;
- one explicit step equals RHS + solve over the whole tensor.

The comparisons over the whole tensor run on the device in slabs.  Under the
bounds-checked library (ADSG_LIBRARY=checked) the run must also record no
out-of-range access."""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

import ads_gb300 as ads
import oracle

pytestmark = pytest.mark.gpu

P, E = 2, 1288
N = E + P  # 1290 per dimension


def _bands():
    """Columns of the 1D mass and stiffness matrices from the oracle's 1D
    heat RHS at dt = 0 and dt = 1 on unit vectors."""
    pr = oracle.Problem([P], [E])
    cache = {}

    def col(c):
        if c not in cache:
            e = np.zeros(N)
            e[c] = 1.0
            m = pr.heat_rhs(e, 0.0)
            cache[c] = (m, m - pr.heat_rhs(e, 1.0))
        return cache[c]

    return col


def _slab_rel_max(a, b, rows=64):
    """max |a - b| / max |b| over (N, N, N) device tensors, a slab at a time."""
    num, den = 0.0, 0.0
    for z in range(0, N, rows):
        x, y = a[z:z + rows], b[z:z + rows]
        num = max(num, float((x - y).abs().max()))
        den = max(den, float(y.abs().max()))
    return num / den


def test_largest_accepted_tensor(cuda, monkeypatch):
    free = torch.cuda.mem_get_info()[0]
    if free < 150e9:
        pytest.skip(f"needs ~120 GB of free device memory, {free / 1e9:.0f} GB free")
    for k, v in (("ADSG_PDL", "0"), ("ADSG_FUSE_X", "0"), ("ADSG_STEP_GRAPHS", "0")):
        monkeypatch.setenv(k, v)  # one launch mode: no launch-mode timing at this size
    dims = [ads.Dimension(P, E) for _ in range(3)]
    ctx = ads.Context(dims)
    assert ctx.size == N ** 3 and ctx.size < 2 ** 31
    gen = torch.Generator(device="cuda").manual_seed(11)
    u = torch.rand(N, N, N, dtype=torch.float64, device="cuda", generator=gen).mul_(2.0).sub_(1.0)
    r = torch.empty_like(u)
    dt = 1e-6
    ctx.heat_rhs(u, r, dt)
    ctx.synchronize()

    # sampled points: corners, band-edge rows, the last dof, and random ones
    rng = np.random.default_rng(7)
    pts = [(0, 0, 0), (N - 1, N - 1, N - 1), (1, N - 2, 2), (N - 3, 0, N - 1), (N // 2, N - 1, 0)]
    pts += [tuple(int(v) for v in rng.integers(0, N, 3)) for _ in range(24)]
    col = _bands()
    worst = 0.0
    for i, j, k in pts:  # x, y, z; the tensor is [z][y][x]
        lo = [max(0, c - P) for c in (i, j, k)]
        hi = [min(N, c + P + 1) for c in (i, j, k)]
        nb = u[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]].cpu().numpy()
        mx, kx = (np.array([col(a)[t][i] for a in range(lo[0], hi[0])]) for t in (0, 1))
        my, ky = (np.array([col(b)[t][j] for b in range(lo[1], hi[1])]) for t in (0, 1))
        mz, kz = (np.array([col(c)[t][k] for c in range(lo[2], hi[2])]) for t in (0, 1))
        w = (np.einsum("c,b,a->cba", mz, my, mx)
             - dt * (np.einsum("c,b,a->cba", mz, my, kx) + np.einsum("c,b,a->cba", mz, ky, mx)
                     + np.einsum("c,b,a->cba", kz, my, mx)))
        want = float((w * nb).sum())
        scale = float((np.abs(w) * np.abs(nb)).sum())
        got = float(r[k, j, i])
        err = abs(got - want) / scale
        worst = max(worst, err)
        assert err <= 1e-13, f"point {(i, j, k)}: {got} against {want}"
    print(f"[parity] 1290^3 RHS at {len(pts)} sampled points: worst {worst:.2e} of the terms' magnitude")

    # the solve inverts the mass apply
    ctx.heat_rhs(u, r, 0.0)
    ctx.ads_solve(r)
    ctx.synchronize()
    e_inv = _slab_rel_max(r, u)
    print(f"[parity] 1290^3 solve of the mass apply: {e_inv:.2e}")
    assert e_inv <= 1e-12

    # one step equals RHS + solve
    ctx.heat_rhs(u, r, dt)
    ctx.ads_solve(r)
    s = u.clone()
    del u
    torch.cuda.empty_cache()
    ctx.heat_steps(s, dt, 1)
    ctx.synchronize()
    e_step = _slab_rel_max(s, r)
    print(f"[parity] 1290^3 step against RHS + solve: {e_step:.2e}")
    assert e_step <= 1e-13
    if os.environ.get("ADSG_LIBRARY") == "checked":
        rep = ads.debug_bounds()
        assert rep["violations"] == 0, rep
    ctx.close()
