"""Parity tolerances.

The contract is relative L2 <= 1e-12 per step and <= 1e-10 after a full run.
Those bounds are attainable as stated when the Kronecker mass matrix is well
conditioned (p <= 2: cond(M_1D) ~ 10).  A step solves M u = rhs, so any two
correct implementations whose RHS differ by rounding (~1e-15 relative, e.g.
the reference's literal heat_3d loop vs its executor form) differ after the
solve by up to cond(M_x (x) M_y (x) M_z) times that.  For p = 3, 4 the product of
the 1D condition numbers reaches 2e4 .. 3.3e5, and the reference disagrees
with itself at the 1e-12 .. 1e-11 level.  The bounds are therefore scaled by
prod(cond_d) / 1e3 when that exceeds one (never loosened for p <= 2 in 2D,
and by at most ~1.2 for p = 2 in 3D).
"""
from __future__ import annotations

import numpy as np


def mass_condition(mass_ab: np.ndarray, p: int) -> float:
    """2-norm condition number of a kl = ku = p mass band (LAPACK layout)."""
    ldab = 3 * p + 1
    n = mass_ab.size // ldab
    ab = mass_ab.reshape(n, ldab)
    M = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - p), min(n, j + p + 1)):
            M[i, j] = ab[j, 2 * p + i - j]
    return float(np.linalg.cond(M))


def scale(conds) -> float:
    return max(1.0, float(np.prod(conds)) / 1e3)


def step_tol(conds) -> float:
    return 1e-12 * scale(conds)


def run_tol(conds) -> float:
    return 1e-10 * scale(conds)
