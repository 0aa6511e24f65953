"""CPU reference adjoint assembled from oracle primitives (test helper)."""
from __future__ import annotations

import numpy as np


def forward(pr, u0, kappa, dt, nsteps):
    us = [np.array(u0, np.float64)]
    for _ in range(nsteps):
        us.append(pr.kappa_step(us[-1], kappa, dt))
    return us


def mass_loss(pr, u, target):
    d = u - target
    md = pr.heat_rhs(d, 0.0)  # dt = 0: the Kronecker mass matrix applied to d
    return float(d @ md), 2.0 * md


def gradients(pr, u0, kappa, dt, nsteps, target):
    us = forward(pr, u0, kappa, dt, nsteps)
    loss, lam = mass_loss(pr, us[-1], target)
    g = np.zeros(pr.size)
    for k in reversed(range(nsteps)):
        mu = pr.ads_solve(lam, trans=True)
        pr.kappa_grad(us[k], mu, dt, g)
        lam = pr.heat_rhs_kappa(mu, kappa, dt)
    return loss, lam, g
