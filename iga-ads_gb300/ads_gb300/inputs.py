"""Seeded synthetic initial fields for the heat benchmarks and tests.

The initial coefficients are the L2 projection of prod_d sin(pi x_d) onto the
spline space (the reference computes projections with compute_projection +
ads_solve, include/ads/projection.hpp:148-153 and heat_3d.hpp:35-36) plus
seeded uniform noise in [-amp, amp] from a counter-based SplitMix64 stream, so
any index of any instance can be regenerated independently.

Because f is a product of 1D functions and the mass matrix is a Kronecker
product, the projection is the outer product of the 1D projections; each 1D
projection is computed here on the host from the dimension's quadrature
tables (set-up work, not the hot path).
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0x9E3779B97F4A7C15)
_M2 = np.uint64(0xBF58476D1CE4E5B9)
_M3 = np.uint64(0x94D049BB133111EB)


def splitmix_uniform(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Uniform [0, 1) doubles: SplitMix64 of (seed, offset + i), i < count."""
    with np.errstate(over="ignore"):
        idx = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + idx * _M1
        z = (z ^ (z >> np.uint64(30))) * _M2
        z = (z ^ (z >> np.uint64(27))) * _M3
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def projection_1d(dim, fun=None) -> np.ndarray:
    """Coefficients of the L2 projection of fun (default sin(pi x)) on one dimension."""
    t = dim.tables()
    p, E, q, n = dim.p, dim.elements, dim.quad_order, dim.dofs()
    b = t["btab"].reshape(E, q, 2, p + 1)
    # quadrature points of every element: x = lerp((X+1)/2, x_e, x_{e+1}); J = (x_{e+1}-x_e)/2
    w = t["w"]
    J = t["J"]
    X = _gauss_nodes(q)
    left = np.concatenate([[0.0], np.cumsum(2.0 * J)])[:-1]
    xq = left[:, None] + (X[None, :] + 1.0) * J[:, None]
    fun = fun or (lambda x: np.sin(np.pi * x))
    f = fun(xq)
    F = np.zeros(n)
    for a in range(p + 1):
        np.add.at(F, t["first_dofs"] + a, (f * b[:, :, 0, a] * w[None, :] * J[:, None]).sum(axis=1))
    M = np.zeros((n, n))
    mb = dim.form_band(0)  # rows = columns j, entries ab[j][kl+ku+i-j]
    kl = ku = p
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            M[i, j] = mb[j, kl + ku + i - j]
    return np.linalg.solve(M, F)


def _gauss_nodes(q: int) -> np.ndarray:
    x, _ = np.polynomial.legendre.leggauss(q)
    return x


def initial_field(dims, seed: int = 0, amp: float = 1e-2) -> np.ndarray:
    """x-fastest tensor: outer product of 1D sin projections + seeded noise."""
    vecs = [projection_1d(d) for d in dims]
    u = vecs[0]
    for v in vecs[1:]:
        u = np.multiply.outer(v, u)  # later dims vary slower
    u = np.ascontiguousarray(u.ravel())
    u += (2.0 * splitmix_uniform(seed, u.size) - 1.0) * amp
    return u


def kappa_field(dims, seed: int = 0, modes: int = 8, amp: float = 0.5) -> np.ndarray:
    """Diffusion-field coefficients 1 + amp * f with f a sum of `modes` seeded
    Fourier modes normalised to max |f| = 1, sampled at the coefficients'
    parametric positions i/(n-1) (x-fastest, like the state)."""
    r = splitmix_uniform(seed, modes * (len(dims) + 2))
    axes = [np.linspace(0.0, 1.0, d.dofs()) for d in dims]
    grids = np.meshgrid(*axes[::-1], indexing="ij")[::-1]  # x varies fastest in the flattened array
    f = np.zeros(grids[0].shape)
    for m in range(modes):
        base = m * (len(dims) + 2)
        phase = 2 * np.pi * r[base]
        weight = 2 * r[base + 1] - 1
        arg = phase
        for d, g in enumerate(grids):
            k = 1 + int(r[base + 2 + d] * 4)  # wave numbers 1..4
            arg = arg + 2 * np.pi * k * g
        f += weight * np.cos(arg)
    f /= max(np.abs(f).max(), 1e-300)
    return np.ascontiguousarray((1.0 + amp * f).ravel())
