"""ctypes bindings of the CPU oracle (ads_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
as the checker; the product (iga-ads_gb300/) never imports it.  The shared
library is built by `make -C oracle oracle` (gcc, no GPU).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libads_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libadsref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "ads_oracle.c")):
            build()
        L = ctypes.CDLL(LIB)
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc_problem_create.restype = vp
        L.orc_problem_create.argtypes = [i, _ip, _ip]
        L.orc_problem_destroy.argtypes = [vp]
        L.orc_problem_dofs.argtypes = [vp, i]
        L.orc_problem_size.restype = ctypes.c_long
        L.orc_problem_size.argtypes = [vp]
        L.orc_problem_dim.argtypes = [vp, i, _dp, _dp, _dp, _ip, _dp, _dp, _ip]
        L.orc_heat_rhs.argtypes = [vp, _dp, _dp, d]
        L.orc_heat_rhs_mt.argtypes = [vp, _dp, _dp, d, i]
        L.orc_heat_rhs_kappa.argtypes = [vp, _dp, _dp, _dp, d]
        L.orc_ads_solve.argtypes = [vp, _dp]
        L.orc_ads_solve_t.argtypes = [vp, _dp]
        L.orc_heat_steps.argtypes = [vp, _dp, d, i, i]
        L.orc_projection_sin.argtypes = [vp, _dp]
        L.orc_kappa_grad.argtypes = [vp, _dp, _dp, _dp, d]
        L.orc_form_rhs.argtypes = [vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_gauss.argtypes = [i, _dp, _dp]
        L.orc_dgbtrf.argtypes = [i, i, i, _dp, i, _ip]
        L.orc_dgbtrs.argtypes = [ctypes.c_char, i, i, i, i, _dp, i, _ip, _dp, i]
        L.orc_form_band.argtypes = [i, i, i, i, _dp, _dp, _dp, _ip, _dp]
        L.orc_basis_tables.argtypes = [i, i, d, d, i, _dp, _dp, _dp, _ip]
        _lib = L
    return _lib


def dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def ip(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class Problem:
    """orc_problem: a 1-3D uniform heat problem with factorised mass matrices."""

    def __init__(self, p, elements):
        p = list(p)
        elements = list(elements)
        self.ndim = len(p)
        self._h = lib().orc_problem_create(self.ndim, ip(np.array(p, np.int32)), ip(np.array(elements, np.int32)))
        if not self._h:
            raise ValueError("orc_problem_create failed")
        self.p = p
        self.elements = elements
        self.shape = tuple(e + q for e, q in zip(elements, p))
        self.size = int(np.prod(self.shape))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_problem_destroy(self._h)
            self._h = None

    def dim(self, d):
        p, E = self.p[d], self.elements[d]
        q, n, ldab = p + 1, E + p, 3 * p + 1
        out = dict(btab=np.zeros(E * q * 2 * (p + 1)), w=np.zeros(q), J=np.zeros(E),
                   first_dofs=np.zeros(E, np.int32), mass=np.zeros(ldab * n), lu=np.zeros(ldab * n),
                   ipiv=np.zeros(n, np.int32))
        lib().orc_problem_dim(self._h, d, dp(out["btab"]), dp(out["w"]), dp(out["J"]), ip(out["first_dofs"]),
                              dp(out["mass"]), dp(out["lu"]), ip(out["ipiv"]))
        return out

    def heat_rhs(self, u_prev, dt, nthreads=1):
        u_prev = np.ascontiguousarray(u_prev, np.float64)
        rhs = np.zeros(self.size)
        if nthreads > 1:
            lib().orc_heat_rhs_mt(self._h, dp(u_prev), dp(rhs), dt, nthreads)
        else:
            lib().orc_heat_rhs(self._h, dp(u_prev), dp(rhs), dt)
        return rhs

    def heat_rhs_kappa(self, u_prev, kappa, dt):
        u_prev = np.ascontiguousarray(u_prev, np.float64)
        kappa = np.ascontiguousarray(kappa, np.float64)
        rhs = np.zeros(self.size)
        lib().orc_heat_rhs_kappa(self._h, dp(u_prev), dp(kappa), dp(rhs), dt)
        return rhs

    def ads_solve(self, rhs, trans=False):
        x = np.array(rhs, np.float64, copy=True, order="C")
        (lib().orc_ads_solve_t if trans else lib().orc_ads_solve)(self._h, dp(x))
        return x

    def heat_steps(self, u, dt, nsteps, nthreads=1):
        x = np.array(u, np.float64, copy=True, order="C")
        lib().orc_heat_steps(self._h, dp(x), dt, nsteps, nthreads)
        return x

    def kappa_grad(self, u, mu, dt, g=None):
        g = np.zeros(self.size) if g is None else g
        lib().orc_kappa_grad(self._h, dp(np.ascontiguousarray(u, np.float64)), dp(np.ascontiguousarray(mu, np.float64)),
                             dp(g), dt)
        return g

    def form_rhs(self, u, alpha=0.0, beta=0.0, gamma=0.0, delta=0.0, alpha_q=None, beta_q=None, gamma_q=None,
                 delta_q=None):
        """General pointwise form of the element loop (orc_form_rhs)."""
        fields = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (alpha_q, beta_q, gamma_q, delta_q)]
        uu = None if u is None else np.ascontiguousarray(u, np.float64)
        cst = np.array([alpha, beta, gamma, delta], np.float64)
        rhs = np.zeros(self.size)
        lib().orc_form_rhs(self._h, None if uu is None else dp(uu), dp(cst),
                           *[None if f is None else dp(f) for f in fields], dp(rhs))
        return rhs

    def kappa_step(self, u, kappa, dt):
        """One step of the kappa-weighted scheme: M^{-1} R(kappa) u."""
        return self.ads_solve(self.heat_rhs_kappa(u, kappa, dt))

    def projection_sin(self):
        out = np.zeros(self.size)
        lib().orc_projection_sin(self._h, dp(out))
        return out


def dgbtrf(n, kl, ku, ab, ldab):
    ab = np.array(ab, np.float64, copy=True, order="C")
    ipiv = np.zeros(n, np.int32)
    info = lib().orc_dgbtrf(n, kl, ku, dp(ab), ldab, ip(ipiv))
    return ab, ipiv, info


def dgbtrs(trans, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb):
    ab = np.ascontiguousarray(ab, np.float64)
    ipiv = np.ascontiguousarray(ipiv, np.int32)
    x = np.array(b, np.float64, copy=True, order="C")
    lib().orc_dgbtrs(trans.encode()[:1], n, kl, ku, nrhs, dp(ab), ldab, ip(ipiv), dp(x), ldb)
    return x


def rel_l2(a, b):
    """Relative L2 difference, scaled to avoid overflow on growing fields."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    s = max(np.abs(a).max(), np.abs(b).max())
    if s == 0:
        return 0.0
    return float(np.linalg.norm((a - b) / s) / max(np.linalg.norm(a / s), 1e-300))
