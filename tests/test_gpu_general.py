"""Generalised ADS (one special direction with a band per grid line) against
the known answers of the reference test tests/ads/solver_test.cpp:257-534, and
against a per-line oracle solve on random data."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

import ads_gb300 as ads
import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _lib():
    L = ads.library()
    L.adsg_line_bands_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _ip,
                                         ctypes.c_longlong, _ip, ctypes.POINTER(ctypes.c_void_p)]
    L.adsg_line_bands_destroy.argtypes = [ctypes.c_void_p]
    L.adsg_ads_solve_general_host.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, _dp]
    return L


def _desc(n, lu, ipiv, kl=1, ku=1, keep=None):
    """Descriptor of a bare factorised band of size n (p = 1 placeholder tables)."""
    E = max(n - 1, 1)
    k = dict(btab=np.full(E * 8, 0.5), w=np.ones(2), J=np.full(E, 0.5), first=np.arange(E, dtype=np.int32),
             lu=np.ascontiguousarray(lu, np.float64), ipiv=np.ascontiguousarray(ipiv, np.int32))
    keep.append(k)
    d = ads.DimDesc()
    d.p, d.elements, d.quad_order, d.n = 1, E, 2, n
    d.btab, d.w, d.J = k["btab"].ctypes.data_as(_dp), k["w"].ctypes.data_as(_dp), k["J"].ctypes.data_as(_dp)
    d.first_dofs = k["first"].ctypes.data_as(_ip)
    d.kl, d.ku, d.ldab = kl, ku, 2 * kl + ku + 1
    d.lu, d.ipiv = k["lu"].ctypes.data_as(_dp), k["ipiv"].ctypes.data_as(_ip)
    return d


def _solve_general(descs, special, mats, line_matrix, rhs, kl=1, ku=1):
    L = _lib()
    keep = []
    arr = (ads.DimDesc * len(descs))(*descs)
    ctx = ctypes.c_void_p()
    ads._check(L.adsg_ctx_create(len(descs), arr, ctypes.byref(ctx)))
    n = descs[special].n
    ldab = 2 * kl + ku + 1
    ab = np.ascontiguousarray(np.concatenate([m[0] for m in mats]), np.float64)
    piv = np.ascontiguousarray(np.concatenate([m[1] for m in mats]), np.int32)
    lm = np.ascontiguousarray(line_matrix, np.int32)
    lb = ctypes.c_void_p()
    ads._check(L.adsg_line_bands_create(n, kl, ku, ldab, len(mats), ab.ctypes.data_as(_dp), piv.ctypes.data_as(_ip),
                                        lm.size, lm.ctypes.data_as(_ip), ctypes.byref(lb)))
    x = np.ascontiguousarray(rhs, np.float64).copy()
    ads._check(L.adsg_ads_solve_general_host(ctx, special, lb, x.ctypes.data_as(_dp)))
    L.adsg_line_bands_destroy(lb)
    L.adsg_ctx_destroy(ctx)
    return x


def test_generalised_2d_known_answers(cuda):
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    keep = []
    A = (g["gen2_lu_A"], g["gen2_ipiv_A"])
    B1, B2 = (g["gen2_lu_B1"], g["gen2_ipiv_B1"]), (g["gen2_lu_B2"], g["gen2_ipiv_B2"])
    dA, dB = _desc(2, *A, keep=keep), _desc(3, *B1, keep=keep)
    # special dim second: sizes {na=2, nb=3}
    x = _solve_general([dA, dB], 1, [B1, B2], [0, 1], g["gen2_rhs_second"])
    np.testing.assert_allclose(x, g["gen2_expected"], rtol=1e-13)
    # special dim first: sizes {nb=3, na=2}
    x = _solve_general([dB, dA], 0, [B1, B2], [0, 1], g["gen2_rhs_first"])
    np.testing.assert_allclose(x, g["gen2_expected"], rtol=1e-13)


@pytest.mark.parametrize("section,special", [("first", 0), ("second", 1), ("third", 2)])
def test_generalised_3d_known_answers(section, special, cuda):
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    keep = []
    A = (g["gen3_lu_A"], g["gen3_ipiv_A"])
    B = (g["gen3_lu_B"], g["gen3_ipiv_B"])
    Cs = [(g["gen3_lu_" + c], g["gen3_ipiv_" + c]) for c in ("C11", "C21", "C31", "C12", "C22", "C32")]
    dA, dB, dC = _desc(3, *A, keep=keep), _desc(2, *B, keep=keep), _desc(4, *Cs[0], keep=keep)
    order = {"first": [dC, dA, dB], "second": [dB, dC, dA], "third": [dA, dB, dC]}[section]
    x = _solve_general(order, special, Cs, list(range(6)), g["gen3_rhs_" + section])
    np.testing.assert_allclose(x, g["gen3_expected"], rtol=1e-12)


@pytest.mark.parametrize("special", [0, 1, 2])
def test_generalised_random_against_oracle(special, cuda):
    rng = np.random.default_rng(special)
    n = (7, 5, 6)
    kl = ku = 2
    ldab = 2 * kl + ku + 1
    mats = []
    for m in range(4):
        ab = np.zeros(ldab * n[special])
        for j in range(n[special]):
            for i in range(max(0, j - ku), min(n[special], j + kl + 1)):
                ab[j * ldab + kl + ku + i - j] = rng.uniform(-1, 1) + (5.0 if i == j else 0.0) * (m % 2 * 2 - 1)
        lu, piv, info = oracle.dgbtrf(n[special], kl, ku, ab, ldab)
        assert info == 0
        mats.append((lu, piv))
    keep = []
    std = []
    for d in range(3):
        ab = np.zeros(ldab * n[d])
        for j in range(n[d]):
            for i in range(max(0, j - ku), min(n[d], j + kl + 1)):
                ab[j * ldab + kl + ku + i - j] = rng.uniform(-1, 1) + (4.0 if i == j else 0.0)
        lu, piv, _ = oracle.dgbtrf(n[d], kl, ku, ab, ldab)
        std.append((lu, piv))
    descs = [_desc(n[d], *std[d], kl=kl, ku=ku, keep=keep) for d in range(3)]
    nlines = int(np.prod(n)) // n[special]
    line_matrix = rng.integers(0, 4, nlines)
    rhs = rng.standard_normal(int(np.prod(n)))
    got = _solve_general(descs, special, mats, line_matrix, rhs, kl=kl, ku=ku)
    # oracle: special direction first with the reference line numbering, then the others cyclically
    t = rhs.reshape(n[::-1]).copy()  # numpy axes (z, y, x)

    def along(arr, d):
        return np.moveaxis(arr, 2 - d, -1)

    a = along(t, special)
    others = [(special + 1) % 3, (special + 2) % 3]
    for idx in np.ndindex(a.shape[:-1]):
        coords = {}
        rest = [dd for dd in (2, 1, 0) if dd != special]  # numpy axis order of the remaining dims
        for dd, v in zip(rest, idx):
            coords[dd] = v
        ref_line = coords[others[0]] + n[others[0]] * coords[others[1]]
        lu, piv = mats[line_matrix[ref_line]]
        a[idx] = oracle.dgbtrs("N", n[special], kl, ku, 1, lu, ldab, piv, a[idx].copy(), n[special])
    for d in others:
        b = along(t, d)
        lu, piv = std[d]
        for idx in np.ndindex(b.shape[:-1]):
            b[idx] = oracle.dgbtrs("N", n[d], kl, ku, 1, lu, ldab, piv, b[idx].copy(), n[d])
    # the shared directions may use the two-ended sweep (rounding differs from dgbtrs)
    assert oracle.rel_l2(got, t.ravel()) <= 1e-12
