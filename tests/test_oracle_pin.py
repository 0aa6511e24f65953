"""Pins the CPU oracle (oracle/ads_oracle.c) against the golden fixtures made
by the reference's own compiled code and against the known answers of the
reference tests (tests/ads/solver_test.cpp, tests/ads/lin/band_solve_test.cpp).
CPU only."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

import oracle
from _tol import RHS, RUN, STEP, check
from conftest import GOLDEN

TABLES = sorted(glob.glob(os.path.join(GOLDEN, "tables_*.npz")))
HEAT = sorted(glob.glob(os.path.join(GOLDEN, "heat_*.npz")))


def _ulp_close(a, b, ulps=8):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.maximum(np.abs(a), np.abs(b)).max()
    return np.abs(a - b).max() <= ulps * np.finfo(np.float64).eps * max(scale, 1e-300)


@pytest.mark.parametrize("path", TABLES, ids=os.path.basename)
def test_tables_match_reference(path):
    g = np.load(path)
    p, E = int(g["p"]), int(g["elements"])
    pr = oracle.Problem([p], [E])
    d = pr.dim(0)
    # basis_data tables and the assembled mass matrix are bit-identical
    np.testing.assert_array_equal(d["btab"], g["btab"])
    np.testing.assert_array_equal(d["w"], g["w"])
    np.testing.assert_array_equal(d["J"], g["J"])
    np.testing.assert_array_equal(d["first_dofs"], g["first_dofs"])
    np.testing.assert_array_equal(d["mass"], g["mass"])
    # dgbtrf: identical pivots, factors within a few ulps (BLAS kernels may fuse)
    np.testing.assert_array_equal(d["ipiv"], g["ipiv"])
    assert _ulp_close(d["lu"], g["lu"])


def test_gauss_rules_are_exact_for_polynomials():
    lib = oracle.lib()
    for q in range(2, 65):
        x = np.zeros(q)
        w = np.zeros(q)
        assert lib.orc_gauss(q, oracle.dp(x), oracle.dp(w)) == 0
        assert abs(w.sum() - 2.0) < 1e-13
        for k in range(0, 2 * q, 2):
            exact = 2.0 / (k + 1)
            assert abs((w * x ** k).sum() - exact) < 1e-12 * max(1, q / 8)
        assert np.all(np.diff(x) > 0)


def test_known_answers_ads_solve_1d_2d_3d():
    """solver_test.cpp:63-255: ADS in 1D/2D/3D with exact integer answers."""
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    for name, n in (("x", 4), ("y", 3), ("z", 2)):
        ab = g["m" + name]
        lu, piv, info = oracle.dgbtrf(n, 1, 1, ab, 4)
        assert info == 0
        np.testing.assert_array_equal(piv, g["ipiv_" + name])
        assert _ulp_close(lu, g["lu_" + name])
    lus = {}
    for name, n in (("x", 4), ("y", 3), ("z", 2)):
        lus[name] = (n, g["lu_" + name], g["ipiv_" + name])

    def solve_dir(t, shape, d):
        n, lu, piv = lus["xyz"[d]]
        t = t.reshape(shape[::-1])  # numpy order: (z, y, x)
        axis = len(shape) - 1 - d
        moved = np.moveaxis(t, axis, -1).copy()
        flat = moved.reshape(-1, n)
        out = np.stack([oracle.dgbtrs("N", n, 1, 1, 1, lu, 4, piv, row, n) for row in flat])
        return np.moveaxis(out.reshape(moved.shape), -1, axis).ravel()

    x = oracle.dgbtrs("N", 4, 1, 1, 1, lus["x"][1], 4, lus["x"][2], g["rhs1"], 4)
    np.testing.assert_allclose(x, g["expected1"], rtol=1e-12)
    x2 = g["rhs2"]
    for d in range(2):
        x2 = solve_dir(x2, (4, 3), d)
    np.testing.assert_allclose(x2, g["expected2"], rtol=1e-12)
    x3 = g["rhs3"]
    for d in range(3):
        x3 = solve_dir(x3, (4, 3, 2), d)
    np.testing.assert_allclose(x3, g["expected3"], rtol=1e-12)


def test_known_answers_band_solve():
    """band_solve_test.cpp:15-46: kl=1, ku=2, n=6, four right-hand sides."""
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    lu, piv, info = oracle.dgbtrf(6, 1, 2, g["band6_ab"], 5)
    assert info == 0
    np.testing.assert_array_equal(piv, g["band6_ipiv"])
    x = oracle.dgbtrs("N", 6, 1, 2, 4, lu, 5, piv, g["band6_b"], 6)
    np.testing.assert_allclose(x, g["band6_expected"], atol=1e-5)  # the reference test's margin
    assert oracle.rel_l2(x, g["band6_ref_x"]) <= 1e-14


def test_transposed_solve_is_the_adjoint():
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    lu, piv, _ = oracle.dgbtrf(6, 1, 2, g["band6_ab"], 5)
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal(6), rng.standard_normal(6)
    xa = oracle.dgbtrs("N", 6, 1, 2, 1, lu, 5, piv, a, 6)
    xb = oracle.dgbtrs("T", 6, 1, 2, 1, lu, 5, piv, b, 6)
    assert abs(xa @ b - a @ xb) < 1e-13 * np.abs(xa @ b)


@pytest.mark.parametrize("path", HEAT, ids=os.path.basename)
def test_heat_step_matches_reference(path):
    g = np.load(path)
    nd, p, E = int(g["ndim"]), int(g["p"]), int(g["elements"])
    dt, N = float(g["dt"]), int(g["nsteps"])
    pr = oracle.Problem([p] * nd, [E] * nd)
    name = os.path.basename(path)
    np.testing.assert_allclose(pr.projection_sin(), g["projection"], rtol=0, atol=1e-15 * np.abs(g["projection"]).max())
    check(f"oracle {name} rhs", oracle.rel_l2(pr.heat_rhs(g["u0"], dt), g["rhs"]), RHS)
    check(f"oracle {name} solve", oracle.rel_l2(pr.ads_solve(g["u0"]), g["solve"]), RHS)
    check(f"oracle {name} 1 step", oracle.rel_l2(pr.heat_steps(g["u0"], dt, 1), g["u1"]), STEP, g["self_u1"])
    check(f"oracle {name} {N} steps", oracle.rel_l2(pr.heat_steps(g["u0"], dt, N), g["uN"]), RUN, g["self_uN"])


@pytest.mark.parametrize("path", HEAT[:3], ids=os.path.basename)
def test_parallel_executor_matches_sequential(path):
    g = np.load(path)
    nd, p, E = int(g["ndim"]), int(g["p"]), int(g["elements"])
    pr = oracle.Problem([p] * nd, [E] * nd)
    a = pr.heat_rhs(g["u0"], float(g["dt"]))
    b = pr.heat_rhs(g["u0"], float(g["dt"]), nthreads=4)
    assert oracle.rel_l2(a, b) <= 1e-14


def test_kappa_one_reduces_to_heat():
    g = np.load(os.path.join(GOLDEN, "heat_3d_p2_e8.npz"))
    pr = oracle.Problem([2] * 3, [8] * 3)
    kappa = np.ones(pr.size)
    a = pr.heat_rhs_kappa(g["u0"], kappa, float(g["dt"]))
    assert oracle.rel_l2(a, g["rhs"]) <= 1e-13


def test_oracle_adjoint_matches_finite_differences():
    """The oracle's adjoint (transposed solves, R(kappa) symmetric, kappa
    gradient assembly) against central differences of the oracle forward."""
    import _adjoint_ref as ar

    pr = oracle.Problem([2, 3], [5, 4])
    rng = np.random.default_rng(4)
    u0 = rng.uniform(-1, 1, pr.size)
    kappa = 1 + 0.3 * rng.uniform(-1, 1, pr.size)
    target = rng.uniform(-1, 1, pr.size)
    dt, N = 2e-3, 4
    L, gu, gk = ar.gradients(pr, u0, kappa, dt, N, target)

    def loss(u, k):
        return ar.mass_loss(pr, ar.forward(pr, u, k, dt, N)[-1], target)[0]

    for seed in range(3):
        d = np.random.default_rng(100 + seed).standard_normal(pr.size)
        h = 1e-5
        fd_u = (loss(u0 + h * d, kappa) - loss(u0 - h * d, kappa)) / (2 * h)
        assert abs(fd_u - gu @ d) <= 1e-7 * max(abs(fd_u), 1e-30)
        fd_k = (loss(u0, kappa + h * d) - loss(u0, kappa - h * d)) / (2 * h)
        assert abs(fd_k - gk @ d) <= 1e-6 * max(abs(fd_k), 1e-30)


def _grid(xq, E, q):
    """Gauss-point coordinates of a cube, x-fastest over (rx, ry, rz)."""
    axis = np.asarray(xq).reshape(E * q)
    z, y, x = np.meshgrid(axis, axis, axis, indexing="ij")
    return x.ravel(), y.ravel(), z.ravel()


def form_fields(g):
    """Point fields of a form fixture: scalability (test3d.hpp:56-63, the
    forcing added without a test function) or flow (flow.hpp:77-98, with the
    recorded permeability and u at the Gauss points, forcing flow.hpp:128-132)."""
    p, E, dt = int(g["p"]), int(g["elements"]), float(g["dt"])
    x, y, z = _grid(g["xq"], E, p + 1)
    if "kq" not in g:
        r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2)
        f = np.exp(-r) + 1 + np.cos(np.pi * x) * np.cos(np.pi * y) * np.cos(np.pi * z)
        return dict(alpha=1.0, beta=-dt, delta_q=dt * f)
    h = 1 + np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)
    return dict(alpha=1.0, beta_q=-dt * g["kq"] * np.exp(10.0 * g["uq"]), gamma_q=dt * h)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "form_*.npz"))), ids=os.path.basename)
def test_form_rhs_matches_reference(path):
    """The oracle's general pointwise form against the reference's
    scalability_3d / flow compute_rhs loops."""
    g = dict(np.load(path))
    p, E = int(g["p"]), int(g["elements"])
    pr = oracle.Problem([p] * 3, [E] * 3)
    got = pr.form_rhs(g["u0"], **form_fields(g))
    assert oracle.rel_l2(got, g["rhs"]) <= 1e-13
