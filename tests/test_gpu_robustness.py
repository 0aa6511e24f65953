"""Paths the heat benchmark grids do not exercise, against dense numpy
references built from the same 1D matrices:

- Dirichlet rows (dimension::fix_dof, src/ads/simulation/dimension.cpp:23-29):
  the fixed rows make M non-symmetric; the two-ended sweep's tables are
  rebuilt from the factors, so every solve variant and the row-scaled step
  must still solve the fixed system;
- descriptors whose band rows are not translates of one symmetric row (an
  element-size grading folded into the Jacobians): the pair-sum passes must
  fall back to the full band wherever a row is not symmetric."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import ads_gb300 as ads
import oracle

pytestmark = pytest.mark.gpu
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _dense_from_lapack(ab, n, p):
    """Dense matrix of a kl = ku = p band in LAPACK layout (columns of 3p+1)."""
    ldab = 3 * p + 1
    ab = np.asarray(ab).reshape(n, ldab)
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - p), min(n, j + p + 1)):
            A[i, j] = ab[j, 2 * p + i - j]
    return A


def _apply_along(x, shape, mats, inverse):
    """(A_z (x) A_y (x) A_x) x or its inverse on an x-fastest tensor."""
    t = np.asarray(x, np.float64).reshape(shape[::-1])
    for axis_from_last, A in enumerate(mats):
        ax = t.ndim - 1 - axis_from_last
        t = np.moveaxis(t, ax, -1)
        t = np.linalg.solve(A, t.reshape(-1, A.shape[0]).T).T.reshape(t.shape) if inverse else t @ A.T
        t = np.moveaxis(t, -1, ax)
    return t.ravel()


def _fixed(A, k, p):
    A = A.copy()
    n = A.shape[0]
    A[k, max(0, k - p):min(n, k + p + 1)] = 0.0
    A[k, k] = 1.0
    return A


@pytest.mark.parametrize("variant", [None, "0", "3", "4", "5", "6", "7"])
def test_fixed_dofs_every_variant(variant, cuda, monkeypatch):
    import torch

    if variant:
        monkeypatch.setenv("ADSG_SOLVE_VARIANT", variant)
    p, E = (2, 2, 2), (14, 11, 9)
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, E)]
    fixes = [(0, 0), (0, dims[0].dofs() - 1), (1, 0), (2, dims[2].dofs() - 1)]
    for d, k in fixes:
        dims[d].fix_dof(k)
    ctx = ads.Context(dims)
    M = [_dense_from_lapack(d.form_band(0), d.dofs(), d.p) for d in dims]
    for d, k in fixes:
        M[d] = _fixed(M[d], k, dims[d].p)
    shape = [d.dofs() for d in dims]
    b = np.random.default_rng(1).uniform(-1, 1, ctx.size)
    x = b.copy()
    ctx.ads_solve_host(x)
    ref = _apply_along(b, shape, M, inverse=True)
    assert oracle.rel_l2(x, ref) <= 1e-12
    # the step path: compute_rhs (unaffected by the fixes) then the fixed solve
    u = torch.from_numpy(b).cuda()
    r, nxt = torch.empty_like(u), torch.empty_like(u)
    ctx.heat_rhs(u, r, 1e-4)
    ctx.heat_step(u, nxt, 1e-4)
    ctx.synchronize()
    ref_step = _apply_along(r.cpu().numpy(), shape, M, inverse=True)
    assert oracle.rel_l2(nxt.cpu().numpy(), ref_step) <= 1e-12


def _graded_desc(p, E, grade, keep):
    """A descriptor of p / E whose element Jacobians follow a grading: the
    bands stay symmetric matrices but their rows are no longer translates."""
    base = ads.Dimension(p, E)
    d0 = base.descriptor()
    q = d0.quad_order
    btab = np.ctypeslib.as_array(d0.btab, shape=(E * q * 2 * (p + 1),)).copy()
    w = np.ctypeslib.as_array(d0.w, shape=(q,)).copy()
    first = np.ctypeslib.as_array(d0.first_dofs, shape=(E,)).copy().astype(np.int32)
    J = np.ctypeslib.as_array(d0.J, shape=(E,)).copy() * (1.0 + grade * np.sin(np.arange(E) * 0.7))
    n = d0.n
    T = btab.reshape(E, q, 2, p + 1)
    Md, Kd = np.zeros((n, n)), np.zeros((n, n))
    for e in range(E):
        f = first[e]
        for k in range(q):
            Md[f:f + p + 1, f:f + p + 1] += np.outer(T[e, k, 0], T[e, k, 0]) * w[k] * J[e]
            Kd[f:f + p + 1, f:f + p + 1] += np.outer(T[e, k, 1], T[e, k, 1]) * w[k] * J[e]
    ldab = 3 * p + 1
    ab = np.zeros(ldab * n)
    for j in range(n):
        for i in range(max(0, j - p), min(n, j + p + 1)):
            ab[j * ldab + 2 * p + i - j] = Md[i, j]
    lu, ipiv, info = oracle.dgbtrf(n, p, p, ab, ldab)
    assert info == 0
    k = dict(btab=btab, w=w, J=J, first=first, lu=lu, ipiv=ipiv, base=base)
    keep.append(k)
    d = ads.DimDesc()
    d.p, d.elements, d.quad_order, d.n = p, E, q, n
    d.btab, d.w, d.J = k["btab"].ctypes.data_as(_dp), k["w"].ctypes.data_as(_dp), k["J"].ctypes.data_as(_dp)
    d.first_dofs = k["first"].ctypes.data_as(_ip)
    d.kl, d.ku, d.ldab = p, p, ldab
    d.lu, d.ipiv = k["lu"].ctypes.data_as(_dp), k["ipiv"].ctypes.data_as(_ip)
    d.xq = None
    return d, Md, Kd


@pytest.mark.parametrize("grade", [0.0, 0.3])
def test_graded_descriptors_rhs_and_step(grade, cuda):
    """Ungraded rows are symmetric in the interior (pair sums used); graded
    ones are not (full band): both must reproduce the Kronecker formula."""
    import torch

    keep = []
    spec = [(2, 20), (3, 15), (2, 12)]
    built = [_graded_desc(p, E, grade, keep) for p, E in spec]
    arr = (ads.DimDesc * 3)(*[b[0] for b in built])
    h = ctypes.c_void_p()
    ads._check(ads.library().adsg_ctx_create(3, arr, ctypes.byref(h)))
    try:
        n = [b[0].n for b in built]
        size = int(np.prod(n))
        u = np.random.default_rng(2).uniform(-1, 1, size)
        dt = 1e-4
        M = [b[1] for b in built]
        K = [b[2] for b in built]
        # rhs = (Mz Ny... ) written as M(x)M(x)M u - dt (K(x)M(x)M + M(x)K(x)M + M(x)M(x)K) u
        rhs = _apply_along(u, n, M, False)
        for d in range(3):
            mats = [K[i] if i == d else M[i] for i in range(3)]
            rhs -= dt * _apply_along(u, n, mats, False)
        ud = torch.from_numpy(u).cuda()
        r, nxt = torch.empty_like(ud), torch.empty_like(ud)
        lib = ads.library()
        ads._check(lib.adsg_heat_rhs(h, ud.data_ptr(), r.data_ptr(), dt))
        ads._check(lib.adsg_heat_step(h, ud.data_ptr(), nxt.data_ptr(), dt))
        ads._check(lib.adsg_ctx_synchronize(h))
        assert oracle.rel_l2(r.cpu().numpy(), rhs) <= 1e-13
        assert oracle.rel_l2(nxt.cpu().numpy(), _apply_along(rhs, n, M, True)) <= 1e-12
    finally:
        ads.library().adsg_ctx_destroy(h)
