"""GPU parity: the CUDA path through the C-ABI against the reference's own
outputs (golden fixtures) and the CPU oracle, plus size-independent
properties at the benchmark sizes.  All tests here need a GB300."""
from __future__ import annotations

import ctypes
import glob
import os

import numpy as np
import pytest

import ads_gb300 as ads
import oracle
from _tol import RHS, RUN, STEP, check, oracle_self
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

HEAT = sorted(glob.glob(os.path.join(GOLDEN, "heat_*.npz")))


def _ctx(nd, p, E):
    dims = [ads.Dimension(p, E) for _ in range(nd)]
    return dims, ads.Context(dims)


@pytest.mark.parametrize("path", HEAT, ids=os.path.basename)
def test_heat_against_reference_golden(path, cuda):
    g = np.load(path)
    nd, p, E = int(g["ndim"]), int(g["p"]), int(g["elements"])
    dt, N = float(g["dt"]), int(g["nsteps"])
    dims, ctx = _ctx(nd, p, E)
    name = os.path.basename(path)
    u0 = np.ascontiguousarray(g["u0"])
    rhs = np.zeros_like(u0)
    ctx.heat_rhs_host(u0, rhs, dt)
    check(f"{name} rhs", oracle.rel_l2(rhs, g["rhs"]), RHS)
    x = u0.copy()
    ctx.ads_solve_host(x)
    check(f"{name} solve", oracle.rel_l2(x, g["solve"]), RHS)
    u1 = u0.copy()
    ctx.heat_steps_host(u1, dt, 1)
    check(f"{name} 1 step", oracle.rel_l2(u1, g["u1"]), STEP, g["self_u1"])
    uN = u0.copy()
    ctx.heat_steps_host(uN, dt, N)
    check(f"{name} {N} steps", oracle.rel_l2(uN, g["uN"]), RUN, g["self_uN"])


@pytest.mark.parametrize("path", HEAT, ids=os.path.basename)
def test_element_quadrature_against_reference_golden(path, cuda):
    import torch

    g = np.load(path)
    nd, p, E = int(g["ndim"]), int(g["p"]), int(g["elements"])
    dims, ctx = _ctx(nd, p, E)
    u = torch.from_numpy(g["u0"]).to(cuda)
    r = torch.empty_like(u)
    ctx.heat_rhs_elem(u, r, float(g["dt"]))
    ctx.synchronize()
    check(f"{os.path.basename(path)} element rhs", oracle.rel_l2(r.cpu().numpy(), g["rhs"]), RHS)


def test_element_quadrature_with_kappa_against_oracle(cuda):
    import torch

    p, E = 2, 7
    dims, ctx = _ctx(3, p, E)
    pr = oracle.Problem([p] * 3, [E] * 3)
    rng = np.random.default_rng(11)
    u = rng.uniform(-1, 1, pr.size)
    kappa = 1.0 + 0.5 * rng.uniform(-1, 1, pr.size)
    ref = pr.heat_rhs_kappa(u, kappa, 1e-3)
    ud, kd = torch.from_numpy(u).to(cuda), torch.from_numpy(kappa).to(cuda)
    r = torch.empty_like(ud)
    ctx.heat_rhs_elem(ud, r, 1e-3, kappa=kd)
    ctx.synchronize()
    assert oracle.rel_l2(r.cpu().numpy(), ref) <= 1e-13


@pytest.mark.parametrize("p,elements", [((2, 2, 2), (7, 5, 6)), ((1, 1, 1), (9, 4, 5)), ((3, 3, 3), (4, 6, 5)),
                                        ((4, 4, 4), (5, 4, 6))])
def test_kappa_at_gauss_points_gives_the_same_rhs(p, elements, cuda):
    """adsg_kappa_points + adsg_heat_rhs_elem_points (kappa evaluated once at
    every element's Gauss points) against adsg_heat_rhs_elem with the
    coefficients: the same bits, and the oracle's kappa RHS."""
    import torch

    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    q = p[0] + 1
    assert ctx.kappa_points_count() == int(np.prod(elements)) * q ** 3
    rng = np.random.default_rng(sum(elements))
    u = rng.uniform(-1, 1, ctx.size)
    kappa = 1.0 + 0.5 * rng.uniform(-1, 1, ctx.size)
    ud, kd = torch.from_numpy(u).to(cuda), torch.from_numpy(kappa).to(cuda)
    r1, r2 = torch.empty_like(ud), torch.empty_like(ud)
    kq = torch.empty(ctx.kappa_points_count(), dtype=torch.float64, device=cuda)
    ctx.heat_rhs_elem(ud, r1, 1e-3, kappa=kd)
    ctx.kappa_points(kd, kq)
    ctx.heat_rhs_elem_points(ud, r2, 1e-3, kq)
    ctx.synchronize()
    assert torch.equal(r1, r2)
    ref = oracle.Problem(list(p), list(elements)).heat_rhs_kappa(u, kappa, 1e-3)
    check(f"kappa points p={p} E={elements}", oracle.rel_l2(r2.cpu().numpy(), ref), 1e-13)


def test_kappa_points_need_a_3d_context(cuda):
    ctx = ads.Context([ads.Dimension(2, 8), ads.Dimension(2, 9)])
    assert ctx.kappa_points_count() == 0
    with pytest.raises(ads.AdsError) as err:  # refused before any device access
        ctx.kappa_points(16, 32)
    assert err.value.code == 1005


def _raw_dim(n, lu, ipiv, kl=1, ku=1):
    """A descriptor for a bare factorised band (basis tables of a p = 1 space
    with n-1 elements; only the solve uses the band)."""
    E = n - 1
    keep = dict(btab=np.full(E * 2 * 2 * 2, 0.5), w=np.ones(2), J=np.full(E, 0.5),
                first=np.arange(E, dtype=np.int32), lu=np.ascontiguousarray(lu, np.float64),
                ipiv=np.ascontiguousarray(ipiv, np.int32))
    d = ads.DimDesc()
    d.p, d.elements, d.quad_order, d.n = 1, E, 2, n
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    d.btab = keep["btab"].ctypes.data_as(dp)
    d.w = keep["w"].ctypes.data_as(dp)
    d.J = keep["J"].ctypes.data_as(dp)
    d.first_dofs = keep["first"].ctypes.data_as(ip)
    d.kl, d.ku, d.ldab = kl, ku, 2 * kl + ku + 1
    d.lu = keep["lu"].ctypes.data_as(dp)
    d.ipiv = keep["ipiv"].ctypes.data_as(ip)
    return d, keep


def _raw_ctx(descs):
    arr = (ads.DimDesc * len(descs))(*descs)
    h = ctypes.c_void_p()
    ads._check(ads.library().adsg_ctx_create(len(descs), arr, ctypes.byref(h)))
    return h


def test_known_answers_ads_solve_1d_2d_3d(cuda):
    """solver_test.cpp:63-255 through adsg_ads_solve_host."""
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    lib = ads.library()
    dx, kx = _raw_dim(4, g["lu_x"], g["ipiv_x"])
    dy, ky = _raw_dim(3, g["lu_y"], g["ipiv_y"])
    dz, kz = _raw_dim(2, g["lu_z"], g["ipiv_z"])
    for descs, rhs, exp in (([dx], "rhs1", "expected1"), ([dx, dy], "rhs2", "expected2"),
                            ([dx, dy, dz], "rhs3", "expected3")):
        h = _raw_ctx(descs)
        b = np.ascontiguousarray(g[rhs], np.float64).copy()
        ads._check(lib.adsg_ads_solve_host(h, b.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        lib.adsg_ctx_destroy(h)
        np.testing.assert_allclose(b, g[exp], rtol=1e-13)


def test_known_answers_dgbtrs_drop_in(cuda):
    """band_solve_test.cpp:15-46 through the LAPACK-signature entry point."""
    g = np.load(os.path.join(GOLDEN, "solver_known_answers.npz"))
    b = g["band6_b"].copy()
    info = ads.dgbtrs("N", 6, 1, 2, 4, g["band6_lu"], 5, g["band6_ipiv"], b, 6)
    assert info == 0
    np.testing.assert_allclose(b, g["band6_expected"], atol=1e-5)
    assert oracle.rel_l2(b, g["band6_ref_x"]) <= 1e-14
    x = g["rhs1"].copy()
    assert ads.dgbtrs("N", 4, 1, 1, 1, g["lu_x"], 4, g["ipiv_x"], x, 4) == 0
    np.testing.assert_allclose(x, g["expected1"], rtol=1e-13)


def test_dgbtrs_pivoted_p4_many_columns_and_ldb(cuda):
    pr = oracle.Problem([4], [36])
    d = pr.dim(0)
    n, ldab, ldb, nrhs = 40, 13, 43, 77
    rng = np.random.default_rng(5)
    b = rng.standard_normal(ldb * nrhs)
    for trans in ("N", "T"):
        ref = oracle.dgbtrs(trans, n, 4, 4, nrhs, d["lu"], ldab, d["ipiv"], b, ldb)
        x = b.copy()
        assert ads.dgbtrs(trans, n, 4, 4, nrhs, d["lu"], ldab, d["ipiv"], x, ldb) == 0
        assert oracle.rel_l2(x, ref) <= 1e-13
        pad = np.ones(ldb, bool)
        pad[:n] = False
        np.testing.assert_array_equal(x.reshape(nrhs, ldb)[:, pad], b.reshape(nrhs, ldb)[:, pad])


@pytest.mark.parametrize("trans", ["N", "T"])
def test_dgbtrs_lines_longer_than_a_shared_memory_tile(trans, cuda):
    """n = 900 (a line longer than a shared-memory tile holds): swept in
    place in global memory, same result as LAPACK's order."""
    pr = oracle.Problem([4], [896])
    d = pr.dim(0)
    n, ldab, ldb, nrhs = 900, 13, 905, 37
    b = np.random.default_rng(6).standard_normal(ldb * nrhs)
    ref = oracle.dgbtrs(trans, n, 4, 4, nrhs, d["lu"], ldab, d["ipiv"], b, ldb)
    x = b.copy()
    assert ads.dgbtrs(trans, n, 4, 4, nrhs, d["lu"], ldab, d["ipiv"], x, ldb) == 0
    check(f"dgbtrs {trans} n=900", oracle.rel_l2(x, ref), RHS)


def test_context_with_a_dimension_above_850_dofs(cuda):
    """A 2D context with 1200 dofs along x: forward and transposed solves
    and steps against the oracle."""
    import torch

    p, elements = (2, 3), (1198, 20)
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    pr = oracle.Problem(list(p), list(elements))
    u = np.random.default_rng(12).uniform(-1, 1, pr.size)
    x = u.copy()
    ctx.ads_solve_host(x)
    check("1200x23 solve", oracle.rel_l2(x, pr.ads_solve(u)), RHS)
    xt = torch.from_numpy(u).cuda()
    ctx.ads_solve_t(xt)
    ctx.synchronize()
    check("1200x23 transposed solve", oracle.rel_l2(xt.cpu().numpy(), pr.ads_solve(u, trans=True)), RHS)
    s = u.copy()
    ctx.heat_steps_host(s, 1e-7, 2)
    check("1200x23 2 steps", oracle.rel_l2(s, pr.heat_steps(u, 1e-7, 2)), 2 * STEP, oracle_self(pr, u, 1e-7, 2))


@pytest.mark.parametrize("p,elements", [
    ((2, 2, 2), (5, 7, 9)),
    ((2, 3, 4), (6, 5, 4)),
    ((4, 4), (33, 1)),
    ((3,), (40,)),
    ((1, 1, 1), (3, 4, 5)),
])
def test_uneven_grids_against_oracle(p, elements, cuda):
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    pr = oracle.Problem(list(p), list(elements))
    rng = np.random.default_rng(sum(elements))
    u = rng.uniform(-1, 1, pr.size)
    dt = 1e-5
    label = f"uneven p={p} E={elements}"
    r = np.zeros_like(u)
    ctx.heat_rhs_host(u, r, dt)
    check(f"{label} rhs", oracle.rel_l2(r, pr.heat_rhs(u, dt)), RHS)
    x = u.copy()
    ctx.ads_solve_host(x)
    check(f"{label} solve", oracle.rel_l2(x, pr.ads_solve(u)), RHS)
    s = u.copy()
    ctx.heat_steps_host(s, dt, 3)
    check(f"{label} 3 steps", oracle.rel_l2(s, pr.heat_steps(u, dt, 3)), STEP * 3, oracle_self(pr, u, dt, 3))


def test_transposed_solve_is_adjoint(cuda):
    import torch

    dims, ctx = _ctx(3, 4, 9)
    rng = np.random.default_rng(2)
    a = torch.from_numpy(rng.standard_normal(ctx.size)).to(cuda)
    b = torch.from_numpy(rng.standard_normal(ctx.size)).to(cuda)
    xa, xb = a.clone(), b.clone()
    ctx.ads_solve(xa)
    ctx.ads_solve_t(xb)
    ctx.synchronize()
    lhs, rhs = float((xa * b).sum()), float((a * xb).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


# --- full-size properties (the 3D p=2 128^3 benchmark grid) ------------------

@pytest.fixture(scope="module")
def big(cuda):
    import torch

    dims, ctx = _ctx(3, 2, 128)
    from ads_gb300 import inputs

    u = torch.from_numpy(inputs.initial_field(dims, seed=1)).to(cuda)
    return dims, ctx, u


def test_full_size_mass_solve_round_trip(big):
    import torch

    dims, ctx, u = big
    Mu = torch.empty_like(u)
    ctx.heat_rhs(u, Mu, 0.0)  # dt = 0: rhs = (Mx (x) My (x) Mz) u
    ctx.ads_solve(Mu)
    ctx.synchronize()
    err = float(torch.linalg.norm(Mu - u) / torch.linalg.norm(u))
    check("130^3 mass then solve round trip", err, RHS)


def test_full_size_linearity_and_determinism(big):
    import torch

    dims, ctx, u = big
    v = torch.roll(u, 7) * 0.5
    r1, r2, r3 = torch.empty_like(u), torch.empty_like(u), torch.empty_like(u)
    ctx.heat_rhs(u, r1, 1e-6)
    ctx.heat_rhs(v, r2, 1e-6)
    w = 2.0 * u - 3.0 * v
    ctx.heat_rhs(w, r3, 1e-6)
    ctx.synchronize()
    lin = float(torch.linalg.norm(r3 - (2.0 * r1 - 3.0 * r2)) / torch.linalg.norm(r3))
    assert lin <= 1e-13
    s1, s2 = u.clone(), u.clone()
    ctx.heat_steps(s1, 1e-6, 4)
    ctx.heat_steps(s2, 1e-6, 4)
    ctx.synchronize()
    assert torch.equal(s1, s2)


def test_full_size_graph_steps_equal_explicit_loop(big):
    """adsg_heat_steps replays adsg_heat_step bitwise; both agree with
    compute_rhs + ads_solve issued as two calls up to rounding (the step path
    feeds the two-ended solves a row-scaled right-hand side)."""
    import torch

    dims, ctx, u = big
    a = u.clone()
    ctx.heat_steps(a, 1e-6, 3)
    b, tb = u.clone(), torch.empty_like(u)
    for _ in range(3):
        ctx.heat_step(b, tb, 1e-6)
        b, tb = tb, b
    c, tc = u.clone(), torch.empty_like(u)
    for _ in range(3):
        ctx.heat_rhs(c, tc, 1e-6)
        ctx.ads_solve(tc)
        c, tc = tc, c
    ctx.synchronize()
    assert torch.equal(a, b)
    assert float(torch.linalg.norm(b - c) / torch.linalg.norm(c)) <= 1e-13


def test_full_size_element_and_factored_rhs_agree(big):
    import torch

    dims, ctx, u = big
    r1, r2 = torch.empty_like(u), torch.empty_like(u)
    ctx.heat_rhs(u, r1, 1e-6)
    ctx.heat_rhs_elem(u, r2, 1e-6)
    ctx.synchronize()
    assert float(torch.linalg.norm(r1 - r2) / torch.linalg.norm(r1)) <= 1e-13


def test_full_size_against_oracle_one_step_sampled(big):
    """One full 130^3 step against the multi-threaded oracle."""
    dims, ctx, u = big
    pr = oracle.Problem([2] * 3, [128] * 3)
    u0 = u.cpu().numpy()
    ref = pr.heat_steps(u0, 1e-6, 1, nthreads=max(1, min(16, os.cpu_count() or 1)))
    got = u0.copy()
    ctx.heat_steps_host(got, 1e-6, 1)
    check("130^3 p=2 1 step vs oracle", oracle.rel_l2(got, ref), STEP)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("p,elements", [
    ((2, 2, 2), (30, 7, 9)),
    ((4, 4, 4), (12, 9, 6)),
    ((3, 3), (50, 33)),
    ((1, 2, 4), (5, 6, 7)),
    ((2,), (200,)),
])
def test_every_solve_variant_against_oracle(variant, p, elements, cuda, monkeypatch):
    """The autotuner's candidates (staged 1/2/4 tiles per block, in-place
    global sweep, two-ended twisted sweep in global memory, staged through
    shared memory or streamed in chunks) each match the oracle's dgbtrs-based
    ADS solve."""
    monkeypatch.setenv("ADSG_SOLVE_VARIANT", str(variant))
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    pr = oracle.Problem(list(p), list(elements))
    rng = np.random.default_rng(variant + 17 * len(p))
    u = rng.uniform(-1, 1, pr.size)
    x = u.copy()
    ctx.ads_solve_host(x)
    label = f"variant {variant} p={p} E={elements}"
    check(f"{label} solve", oracle.rel_l2(x, pr.ads_solve(u)), RHS)
    s = u.copy()
    ctx.heat_steps_host(s, 1e-5, 2)
    check(f"{label} 2 steps", oracle.rel_l2(s, pr.heat_steps(u, 1e-5, 2)), STEP * 2, oracle_self(pr, u, 1e-5, 2))
    chosen = ctx.solve_variants()
    assert all(0 <= v <= 7 for v in chosen)
    if variant in (0, 3):  # always applicable for p <= 4; a forced variant rules the step's view too
        assert chosen == [variant] * len(p)
        assert ctx.step_solve_variants() == chosen
    if variant in (4, 5, 6, 7):  # the twisted sweeps need n >= 4p + 2 along the direction
        for d, v in zip(dims, chosen):
            assert (v == variant) == (d.dofs() >= 4 * d.p + 2)


def test_failure_detection_counts_nonfinite(cuda):
    """An unstable dt drives the explicit step to overflow; the device count of
    non-finite coefficients reports it (failure made on the host side: only
    the data diverges, no kernel misbehaves)."""
    import torch

    dims, ctx = _ctx(2, 4, 24)
    u = torch.from_numpy(np.random.default_rng(0).uniform(-1, 1, ctx.size)).cuda()
    assert ctx.count_nonfinite(u) == 0
    u[5] = float("nan")
    u[7] = float("inf")
    assert ctx.count_nonfinite(u) == 2
    v = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, ctx.size)).cuda()
    ctx.heat_steps(v, 1e-1, 400)  # far above the stability limit
    ctx.synchronize()
    assert ctx.count_nonfinite(v) > 0


@pytest.mark.parametrize("p,elements", [((2, 2, 2), (20, 18, 16)), ((2, 2), (32, 32)), ((4, 3), (30, 20)),
                                        ((3,), (64,)), ((4, 4), (25, 14)), ((1, 1), (40, 9))])
def test_launch_mode_does_not_change_results(p, elements, cuda, monkeypatch):
    """Programmatic dependent launch only moves when the next kernel's blocks
    are scheduled, and the one-launch 2D step (on one block or on a
    thread-block cluster) runs the separate kernels' operations in the same
    order: those modes agree bitwise.  The fused x
    pass + x solve solves x first (the others solve x last), so the fused
    modes agree bitwise among themselves and with the rest to rounding."""
    out = []
    for pdl, fuse, one, cluster in (("0", "0", "0", "0"), ("1", "0", "0", "0"), ("0", "1", "0", "0"),
                                    ("1", "1", "0", "0"), ("0", "0", "1", "0"), ("1", "0", "1", "0"),
                                    ("0", "0", "1", "1"), ("1", "0", "1", "1")):
        monkeypatch.setenv("ADSG_PDL", pdl)
        monkeypatch.setenv("ADSG_FUSE_X", fuse)
        monkeypatch.setenv("ADSG_STEP_1BLOCK", one)
        monkeypatch.setenv("ADSG_STEP_CLUSTER", cluster)
        monkeypatch.setenv("ADSG_SOLVE_VARIANT", "5")
        dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
        ctx = ads.Context(dims)
        assert ctx.launch_pdl() == (pdl == "1")
        assert ctx.fused_x() == (fuse == "1" and one == "0")
        assert ctx.step_1block() == (one == "1" and len(p) == 2 and p[0] == p[1])
        assert ctx.step_cluster() == (ctx.step_1block() and cluster == "1")
        u = np.random.default_rng(3).uniform(-1, 1, ctx.size)
        ctx.heat_steps_host(u, 1e-5, 5)
        r = np.empty_like(u)
        ctx.heat_rhs_host(u, r, 1e-5)
        out.append((fuse == "1" and ctx.fused_x(), u, r))
    plain = [o for o in out if not o[0]]
    fused = [o for o in out if o[0]]
    for group in (plain, fused):
        for _, u, r in group[1:]:
            np.testing.assert_array_equal(u, group[0][1])
            np.testing.assert_array_equal(r, group[0][2])
    pr = oracle.Problem(list(p), list(elements))
    u0 = np.random.default_rng(3).uniform(-1, 1, pr.size)
    tol_self = oracle_self(pr, u0, 1e-5, 5)
    for _, u, r in fused:
        check(f"fused x p={p} E={elements} 5 steps", oracle.rel_l2(u, plain[0][1]), STEP * 5, tol_self)
        check(f"fused x p={p} E={elements} rhs", oracle.rel_l2(r, plain[0][2]), STEP * 5, tol_self)


@pytest.mark.parametrize("p,elements", [
    ((2, 2, 2), (30, 7, 9)),
    ((4, 4, 4), (12, 9, 6)),
    ((3, 3), (50, 33)),
    ((1, 2, 4), (5, 6, 7)),
    ((2,), (200,)),
    ((3, 2), (1, 40)),
])
def test_heat_step_against_oracle(p, elements, cuda):
    """adsg_heat_step (heat_3d::step) on mixed grids: directions with and
    without the two-ended solve (and so with and without the row-scaled
    right-hand side) against the oracle's compute_rhs + dgbtrs solve."""
    import torch

    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    pr = oracle.Problem(list(p), list(elements))
    u0 = np.random.default_rng(11).uniform(-1, 1, pr.size)
    a = torch.from_numpy(u0).cuda()
    b = torch.empty_like(a)
    for _ in range(2):
        ctx.heat_step(a, b, 1e-5)
        a, b = b, a
    ctx.synchronize()
    check(f"heat_step p={p} E={elements} 2 steps", oracle.rel_l2(a.cpu().numpy(), pr.heat_steps(u0, 1e-5, 2)),
          STEP * 2, oracle_self(pr, u0, 1e-5, 2))
    with pytest.raises(RuntimeError, match="overlap"):
        ctx.heat_step(a, a, 1e-5)


@pytest.mark.parametrize("p,elements,variant", [
    ((2, 2, 2), (30, 7, 9), None),
    ((2, 2, 2), (62, 62, 62), None),
    ((2, 2, 2), (300, 300, 1), None),     # 3 rows along the outermost axis (shorter than a column segment)
    ((4, 4, 4), (60, 60, 60), "3"),
    ((3, 4), (600, 45), None),
    ((1, 1, 1), (40, 30, 50), None),
])
@pytest.mark.parametrize("nsteps", [1, 3])
@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("graphs", ["0", "1"])
def test_host_entry_reading_pinned_input_is_exact(p, elements, variant, nsteps, pinned, graphs, cuda, monkeypatch):
    """adsg_heat_steps_host: from pinned buffers the first band pass reads the
    input in host memory directly (column sweeps); from pageable ones the
    input is copied first; with graph replay on, pinned buffers replay a
    cached graph of the whole call (the second call here).  Every way the
    result equals the device-resident steps bitwise."""
    import torch

    if variant:
        monkeypatch.setenv("ADSG_SOLVE_VARIANT", variant)
    monkeypatch.setenv("ADSG_STEP_GRAPHS", graphs)
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    assert ctx.step_graphs() == (graphs == "1")
    u0 = np.random.default_rng(5).uniform(-1, 1, ctx.size)
    if pinned:
        ht = torch.from_numpy(u0.copy()).pin_memory()
        h = ht.numpy()
    else:
        h = u0.copy()
    d = torch.from_numpy(u0).cuda()
    for _ in range(2):
        ctx.heat_steps_host(h, 1e-5, nsteps)
        ctx.heat_steps(d, 1e-5, nsteps)
        ctx.synchronize()
        np.testing.assert_array_equal(h, d.cpu().numpy())


def test_step_graph_cache_matches_direct_launches(cuda, monkeypatch):
    """adsg_heat_step replays a cached single-step graph per (prev, next, dt);
    with stage timers on it launches directly.  Same kernels: bitwise equal,
    also across dt changes (the dt bands are rebuilt in place before a replay)
    and after the cache has evicted entries."""
    import torch

    monkeypatch.setenv("ADSG_STEP_GRAPHS", "1")
    ctx = ads.Context([ads.Dimension(2, 20), ads.Dimension(3, 14), ads.Dimension(2, 9)])
    assert ctx.step_graphs()
    rng = np.random.default_rng(21)
    bufs = [torch.from_numpy(rng.uniform(-1, 1, ctx.size)).cuda() for _ in range(6)]

    def run(timers):
        ctx.enable_stage_timers(timers)
        outs = []
        for k in range(12):
            src, dst = bufs[k % 3], bufs[3 + (k * 7) % 3]
            dt = (1e-4, 3e-5)[k % 2]
            ctx.heat_step(src, dst, dt)
            ctx.synchronize()
            outs.append(dst.cpu().numpy().copy())
        ctx.enable_stage_timers(False)
        return outs

    a, b, c = run(False), run(True), run(False)
    for x, y, z in zip(a, b, c):
        np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(x, z)


@pytest.mark.parametrize("p,elements", [((2, 2, 2), (40, 33, 20)), ((4, 4, 4), (30, 20, 18)), ((3, 2), (70, 45))])
def test_step_view_takes_its_own_variant(p, elements, cuda, monkeypatch):
    """Unforced, the explicit step keeps ads_solve's variant per direction or,
    where that is LAPACK-order (0-3), may take a two-ended one (4-6) on its
    row-scaled tables; either way the step matches the oracle."""
    import torch

    monkeypatch.delenv("ADSG_SOLVE_VARIANT", raising=False)
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    plain, step = ctx.solve_variants(), ctx.step_solve_variants()
    for a, b in zip(plain, step):
        assert a == b or (a <= 3 and b in (4, 5, 6, 7))
    pr = oracle.Problem(list(p), list(elements))
    u = np.random.default_rng(9).uniform(-1, 1, pr.size)
    ud = torch.from_numpy(u).cuda()
    nxt = torch.empty_like(ud)
    ctx.heat_step(ud, nxt, 1e-5)
    ctx.synchronize()
    check(f"step view p={p} E={elements} 1 step", oracle.rel_l2(nxt.cpu().numpy(), pr.heat_steps(u, 1e-5, 1)), STEP,
          oracle_self(pr, u, 1e-5, 1))


@pytest.mark.parametrize("p,elements", [((2, 2, 2), (40, 33, 20)), ((4, 4, 4), (30, 20, 18)), ((3, 3), (70, 45))])
def test_twisted_variants_agree_bitwise(p, elements, cuda, monkeypatch):
    """The two-ended sweep in global memory (4), with whole lines staged in
    shared memory (5), streamed in 32-row chunks (6) and staged by bulk copies
    of the copy engine (7) perform the same operations in the same order:
    identical results, plain and row-scaled."""
    import torch

    out = []
    for v in ("4", "5", "6", "7"):
        monkeypatch.setenv("ADSG_SOLVE_VARIANT", v)
        ctx = ads.Context([ads.Dimension(pp, e) for pp, e in zip(p, elements)])
        assert ctx.solve_variants() == [int(v)] * len(p)
        u = np.random.default_rng(4).uniform(-1, 1, ctx.size)
        x = u.copy()
        ctx.ads_solve_host(x)
        ud = torch.from_numpy(u).cuda()
        nxt = torch.empty_like(ud)
        ctx.heat_step(ud, nxt, 1e-5)
        ctx.synchronize()
        out.append((x, nxt.cpu().numpy()))
    for x, s in out[1:]:
        np.testing.assert_array_equal(x, out[0][0])
        np.testing.assert_array_equal(s, out[0][1])


@pytest.mark.parametrize("p,elements", [((2, 2, 2), (70, 66, 74)), ((4, 4, 4), (60, 60, 60)), ((2, 3), (700, 400))])
@pytest.mark.parametrize("chunks", ["1", "3", "4"])
@pytest.mark.parametrize("graphs", ["0", "1"])
def test_host_entry_slab_chunks_are_exact(p, elements, chunks, graphs, cuda, monkeypatch):
    """adsg_heat_steps_host on pinned buffers runs the first step's passes and
    the last step's slab-local solves in chunks of outer-axis slabs on two
    streams (ADSG_HOST_CHUNKS; 1 = unchunked).  Every output and line takes
    the same operations, so 1 and 2 steps equal the device-resident steps
    bitwise for every chunk count, with and without graph replay."""
    import torch

    monkeypatch.setenv("ADSG_HOST_CHUNKS", chunks)
    monkeypatch.setenv("ADSG_STEP_GRAPHS", graphs)
    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    assert ctx.size >= 1 << 18  # the direct host-reading path
    u0 = np.random.default_rng(8).uniform(-1, 1, ctx.size)
    for nsteps in (1, 2):
        h = torch.from_numpy(u0.copy()).pin_memory()
        d = torch.from_numpy(u0).cuda()
        ctx.heat_steps_host(h.numpy(), 1e-6, nsteps)
        ctx.heat_steps(d, 1e-6, nsteps)
        ctx.synchronize()
        np.testing.assert_array_equal(h.numpy(), d.cpu().numpy())
