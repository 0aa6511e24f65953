"""Generates the golden fixtures in this folder from the reference's OWN code.

Run in a container where the reference sources are present:
    make -C oracle ref           # builds oracle/_ref/libadsref.so from them
    python tests/golden/make_golden.py          # the small cases
    python tests/golden/make_golden.py --runs   # the full-size runs (hours)
    python tests/golden/make_golden.py --runs-self run_3d_p4_e256 4
                                                # their first step on another thread count

Every output array below is produced by the reference implementation
(oracle/_ref: the reference's src/ads/*.cpp and headers compiled as they lie,
driven through their own classes -- ads::dimension, simulation_2d/3d,
ads_solve, lin::factorize/solve_with_factorized).  Initial fields are the
reference's projection of prod sin(pi x_d) solved by its ads_solve, plus
SplitMix64 noise (the same generator as ads_gb300.inputs.splitmix_uniform).

The norms_* fixtures come from basic_simulation_2d/3d's normL2 / normH1 /
errorL2 / errorH1 (include/ads/simulation/basic_simulation_3d.hpp:281-397);
validation_2d_p2_e16 from the reference's examples/validation class (Dirichlet
on every side, exact solution) and heat2d_dirichlet_p2_e32 from its
examples/heat/heat_2d class (the Dirichlet row at x = 0), both run as they
are (their file output stubbed out).

The form_* fixtures come from the reference's scalability_3d::compute_rhs
(examples/scalability/test3d.hpp:66-95) and flow::compute_rhs
(examples/flow/flow.hpp:77-98, permeability from its own environment class),
reproduced loop for loop on simulation_3d by oracle/ref_driver.cpp.

The small systems in solver_known_answers are those of the reference tests
tests/ads/solver_test.cpp:63-255 and tests/ads/lin/band_solve_test.cpp:15-46,
with the answers those tests expect.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libadsref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def dp(a):
    return a.ctypes.data_as(_dp)


def ip(a):
    return a.ctypes.data_as(_ip)


def splitmix_uniform(seed, count):
    m1, m2, m3 = np.uint64(0x9E3779B97F4A7C15), np.uint64(0xBF58476D1CE4E5B9), np.uint64(0x94D049BB133111EB)
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * m1
        z = (z ^ (z >> np.uint64(30))) * m2
        z = (z ^ (z >> np.uint64(27))) * m3
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def load_ref():
    if not os.path.exists(REF_LIB):
        sys.exit(f"{REF_LIB} missing: run `make -C oracle ref` where the reference sources are present")
    L = ctypes.CDLL(REF_LIB)
    i, d = ctypes.c_int, ctypes.c_double
    L.ref_dim_tables.argtypes = [i, i, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _ip]
    L.ref_stiffness.argtypes = [i, i, _dp]
    L.ref_band_solve.argtypes = [i, i, i, _dp, i, _dp, _dp, _ip]
    L.ref_ads_solve.argtypes = [i, i, i, _dp]
    L.ref_heat_steps.argtypes = [i, i, i, d, i, _dp, i]
    L.ref_heat_rhs.argtypes = [i, i, i, d, _dp, _dp]
    L.ref_projection_sin.argtypes = [i, i, i, _dp]
    L.ref_form_rhs.argtypes = [i, i, i, d, _dp, _dp, _dp, _dp]
    return L


def tables(L, p, E):
    q, n, ldab = p + 1, E + p, 3 * p + 1
    out = dict(btab=np.zeros(E * q * 2 * (p + 1)), xq=np.zeros(E * q), w=np.zeros(q), J=np.zeros(E),
               first_dofs=np.zeros(E, np.int32), mass=np.zeros(ldab * n), lu=np.zeros(ldab * n),
               ipiv=np.zeros(n, np.int32), stiffness=np.zeros(ldab * n))
    info = L.ref_dim_tables(p, E, dp(out["btab"]), dp(out["xq"]), dp(out["w"]), dp(out["J"]), ip(out["first_dofs"]),
                            dp(out["mass"]), dp(out["lu"]), ip(out["ipiv"]))
    assert info == 0
    L.ref_stiffness(p, E, dp(out["stiffness"]))
    out["p"] = np.int32(p)
    out["elements"] = np.int32(E)
    return out


def band_from_rows(kl, ku, n, rows):
    """band_matrix{kl, ku, n} filled as make_matrix (solver_test.cpp:31-41)."""
    ldab = 2 * kl + ku + 1
    ab = np.zeros(ldab * n)
    for i, r in enumerate(rows):
        j = max(i - kl, 0)
        for v in r:
            ab[j * ldab + kl + ku + i - j] = v
            j += 1
    return ab


def known_answers(L):
    out = {}
    # tests/ads/solver_test.cpp:63-99 ("ADS one dimension") and the x matrix of :101-255
    mx = band_from_rows(1, 1, 4, [[1, 2], [2, 3, 1], [-1, 4], [1, 3]])
    my = band_from_rows(1, 1, 3, [[2, 3], [1, 2, -3], [2, 2]])
    mz = band_from_rows(1, 1, 2, [[1, 2], [3, 4]])
    out["mx"], out["my"], out["mz"] = mx, my, mz
    rhs1 = np.array([5.0, 11, 10, 15])
    rhs2 = np.array([61.0, 127, 86, 123, -48, -96, -48, -64, 92, 188, 112, 156])
    rhs3 = np.array([543.0, 1101, 618, 849, -144, -288, -144, -192, 564, 1140, 624, 852,
                     1147, 2329, 1322, 1821, -336, -672, -336, -448, 1220, 2468, 1360, 1860])
    out["rhs1"], out["rhs2"], out["rhs3"] = rhs1, rhs2, rhs3
    out["expected1"] = np.arange(1.0, 5.0)
    out["expected2"] = np.arange(1.0, 13.0)
    out["expected3"] = np.arange(1.0, 25.0)
    # factorise with the reference and solve direction by direction as ads_solve does
    for name, (a, n) in dict(x=(mx, 4), y=(my, 3), z=(mz, 2)).items():
        lu = np.zeros_like(a)
        piv = np.zeros(n, np.int32)
        b = np.zeros(n)
        assert L.ref_band_solve(1, 1, n, dp(a), 1, dp(b), dp(lu), ip(piv)) == 0
        out["lu_" + name], out["ipiv_" + name] = lu, piv
    x = rhs1.copy()
    assert L.ref_band_solve(1, 1, 4, dp(mx), 1, dp(x), None, None) == 0
    out["ref_solution1"] = x
    # tests/ads/lin/band_solve_test.cpp:15-46: kl=1, ku=2, n=6, 4 right-hand sides
    kl, ku, n, d = 1, 2, 6, 4
    ldab = 2 * kl + ku + 1
    ab = np.zeros(ldab * n)
    for i in range(n):
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            ab[j * ldab + kl + ku + i - j] = (i + 1) * 10 + j + 1
    b = np.zeros(n * d)  # column-major n x d
    for i in range(n):
        for j in range(d):
            b[j * n + i] = (j + 1) * (i + 1)
    sol = np.array([0.230377, -0.126052, -0.0016554, -0.00111222, 0.203603, -0.109609])
    out["band6_ab"] = ab.copy()
    out["band6_b"] = b.copy()
    out["band6_expected"] = np.concatenate([(j + 1) * sol for j in range(d)])
    lu = np.zeros_like(ab)
    piv = np.zeros(n, np.int32)
    x = b.copy()
    assert L.ref_band_solve(kl, ku, n, dp(ab), d, dp(x), dp(lu), ip(piv)) == 0
    out["band6_lu"], out["band6_ipiv"], out["band6_ref_x"] = lu, piv, x

    # generalised ADS, tests/ads/solver_test.cpp:257-534: per-line bands along a
    # special dimension; factorised here by the reference's lin::factorize
    def fact(rows, n):
        ab = band_from_rows(1, 1, n, rows)
        lu = np.zeros_like(ab)
        pv = np.zeros(n, np.int32)
        assert L.ref_band_solve(1, 1, n, dp(ab), 0, dp(np.zeros(n)), dp(lu), ip(pv)) == 0
        return lu, pv

    g2 = {"A": ([[1, 2], [3, 4]], 2), "B1": ([[2, 3], [1, 2, -3], [2, 2]], 3), "B2": ([[1, 2], [3, 1, 2], [2, -1]], 3)}
    g3 = {"A": ([[2, 3], [1, 2, -3], [2, 2]], 3), "B": ([[1, 2], [3, 4]], 2),
          "C11": ([[1, 2], [2, 3, 1], [1, -4, 0], [1, 3]], 4), "C21": ([[1, 3], [2, -2, 1], [3, -2, 1], [1, 1]], 4),
          "C31": ([[3, 0], [1, 2, 1], [2, -1, 3], [3, 1]], 4), "C12": ([[2, 3], [-1, 3, 2], [2, 4, 1], [-2, 1]], 4),
          "C22": ([[-1, -2], [3, 2, 1], [2, -1, 1], [1, 1]], 4), "C32": ([[2, 1], [-1, 3, 2], [4, 2, 1], [-3, 2]], 4)}
    for pre, table in (("gen2_", g2), ("gen3_", g3)):
        for name, (rows, n) in table.items():
            lu, pv = fact(rows, n)
            out[pre + "lu_" + name], out[pre + "ipiv_" + name] = lu, pv
    # right-hand sides of the sections, x-fastest, and their expected solutions
    out["gen2_rhs_second"] = np.array([43.0, 61, -24, 136, 56, 11])    # sizes {na=2, nb=3}, special = 1
    out["gen2_rhs_first"] = np.array([54.0, -12, 54, 71, 149, 19])     # sizes {nb=3, na=2}, special = 0
    out["gen2_expected"] = np.arange(1.0, 7.0)
    out["gen3_rhs_first"] = np.array([543.0, 1101, -618, 849, -192, -48, -96, -96, 540, 768, 828, 828,
                                      1900, 1681, 2968, -394, 336, -672, -224, -224, 1192, 1748, 3024, -388])
    out["gen3_rhs_second"] = np.array([351.0, 1325, 732, 1382, -501, 2471, 718, -293, -384, 672, -96, -1344,
                                       -192, -448, -192, -448, 492, 1196, 752, 1912, 872, 3276, 872, -380])
    out["gen3_rhs_third"] = np.array([342.0, -48, 162, 1210, 84, 522, 774, -12, 504, 1934, -168, 1648,
                                      -792, -24, 864, 3542, -56, 2674, 1206, -24, 864, -326, -56, -118])
    out["gen3_expected"] = np.arange(1.0, 25.0)
    return out


def rel_l2(a, b):
    s = max(np.abs(a).max(), np.abs(b).max())
    return float(np.linalg.norm((a - b) / s) / max(np.linalg.norm(a / s), 1e-300)) if s else 0.0


def self_disagreement(L, nd, p, E, dt, nsteps, u0, mode, u1, uN, trials=6):
    """How far the reference's own correct forms of the same step fall from
    the fixture's: the literal heat_3d loop against the executor form (3D)
    and the executor on several threads (galois_executor stand-in: the
    scatter order, and so the rounding, changes from run to run) against the
    sequential one; the largest relative L2 difference over all of them,
    after 1 and after nsteps steps.  Also the solve's sensitivity to its
    input's last bit: the reference's ads_solve of u0 with every entry moved
    by up to one ulp, against that of u0."""
    L.ref_heat_steps_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp,
                                    ctypes.c_int]
    d1 = dN = 0.0
    forms = [("mt", t) for t in range(trials)]
    if nd == 3:
        forms.append(("literal" if mode == 0 else "executor", 0))
    for form, t in forms:
        a, b = u0.copy(), u0.copy()
        if form == "mt":
            L.ref_heat_steps_mt(nd, p, E, dt, 1, dp(a), 2 + t)
            L.ref_heat_steps_mt(nd, p, E, dt, nsteps, dp(b), 2 + t)
        else:
            other = 1 if form == "literal" else 0
            L.ref_heat_steps(nd, p, E, dt, 1, dp(a), other)
            L.ref_heat_steps(nd, p, E, dt, nsteps, dp(b), other)
        d1, dN = max(d1, rel_l2(a, u1)), max(dN, rel_l2(b, uN))
    rng = np.random.default_rng(1234)
    x = u0 * (1.0 + rng.uniform(-1, 1, u0.size) * 2.0 ** -53)
    y = u0.copy()
    L.ref_ads_solve(nd, p, E, dp(x))
    L.ref_ads_solve(nd, p, E, dp(y))
    return dict(self_u1=np.float64(d1), self_uN=np.float64(dN), solve_ulp_sensitivity=np.float64(rel_l2(x, y)))


def heat_case(L, nd, p, E, dt, nsteps, seed, mode=0):
    n = E + p
    size = n ** nd
    u0 = np.zeros(size)
    L.ref_projection_sin(nd, p, E, dp(u0))
    proj = u0.copy()
    L.ref_ads_solve(nd, p, E, dp(u0))
    u0 += (2.0 * splitmix_uniform(seed, size) - 1.0) * 1e-2
    rhs = np.zeros(size)
    L.ref_heat_rhs(nd, p, E, dt, dp(u0), dp(rhs))
    sol = u0.copy()
    L.ref_ads_solve(nd, p, E, dp(sol))
    u1 = u0.copy()
    L.ref_heat_steps(nd, p, E, dt, 1, dp(u1), mode)
    uN = u0.copy()
    L.ref_heat_steps(nd, p, E, dt, nsteps, dp(uN), mode)
    out = dict(ndim=np.int32(nd), p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), nsteps=np.int32(nsteps),
               seed=np.int64(seed), mode=np.int32(mode), projection=proj, u0=u0, rhs=rhs, solve=sol, u1=u1, uN=uN)
    out.update(self_disagreement(L, nd, p, E, dt, nsteps, u0, mode, u1, uN))
    return out


CASES = [
    # (ndim, p, elements, dt, nsteps, seed, mode)
    (2, 2, 32, 1e-5, 100, 1, 0),   # the 2D heat configuration: 34x34 dofs, 100 steps
    (2, 4, 10, 1e-5, 10, 2, 0),
    (3, 2, 4, 1e-6, 3, 3, 1),      # literal heat_3d::compute_rhs
    (3, 2, 8, 1e-6, 10, 4, 0),
    (3, 3, 6, 1e-6, 5, 5, 0),
    (3, 4, 8, 1e-6, 5, 6, 0),      # p = 4: pivoted band LU
    (3, 2, 16, 1e-6, 3, 7, 0),
]


def form_case(L, which, p, E, dt, seed):
    """scalability_3d (which 0) or flow (which 1) compute_rhs from a seeded
    u_prev; flow also records k and u at every Gauss point."""
    n = E + p
    size = n ** 3
    u0 = (2.0 * splitmix_uniform(seed, size) - 1.0) * (0.05 if which else 1.0)
    npts = (E * (p + 1)) ** 3
    rhs, kq, uq = np.zeros(size), np.zeros(npts), np.zeros(npts)
    L.ref_form_rhs(which, p, E, dt, dp(u0), dp(rhs), dp(kq), dp(uq))
    xq = tables(L, p, E)["xq"]
    out = dict(p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), seed=np.int64(seed), u0=u0, rhs=rhs, xq=xq)
    if which:
        out.update(kq=kq, uq=uq)
    return out


FORM_CASES = [
    # (name, which, p, elements, dt, seed)
    ("form_scalability_p2_e5", 0, 2, 5, 1e-4, 11),
    ("form_scalability_p3_e4", 0, 3, 4, 1e-4, 12),
    ("form_flow_p2_e6", 1, 2, 6, 1e-3, 13),
    ("form_flow_p4_e3", 1, 4, 3, 1e-3, 14),
]


# Full-size runs of the 3D configurations: 130^3 dofs p=2 for 50 steps at
# dt=1e-6, and 260^3 dofs p=4 for 20 steps at dt=1e-6 (unstable at that dt:
# its top modes grow ~16.6x per step).  The reference runs them with its
# element loop on the galois_executor stand-in (all host threads); the fixture
# keeps whole planes of the state after the first and the last step plus
# global statistics, since the full fields (17.6 / 140.6 MB) do not belong in
# the repository.  The initial field is ads_gb300.inputs.initial_field (the
# sin projection plus SplitMix64 noise, seed 0), which the GPU test recreates.
RUNS = [
    # (name, p, elements, dt, nsteps, seed)
    ("run_3d_p2_e128", 2, 128, 1e-6, 50, 0),
    ("run_3d_p4_e256", 4, 256, 1e-6, 20, 0),
]


def mass_apply(u, shape, bands):
    """(Mz (x) My (x) Mx) u for an x-fastest tensor, from LAPACK-layout bands."""
    v = u.reshape(shape[::-1])
    for axis, (ab, p) in zip((2, 1, 0), bands):
        n = shape[2 - axis]
        ldab = 3 * p + 1
        M = np.zeros((n, n))
        for j in range(n):
            for i in range(max(0, j - p), min(n, j + p + 1)):
                M[i, j] = ab[j * ldab + 2 * p + i - j]
        v = np.moveaxis(np.tensordot(M, np.moveaxis(v, axis, 0), axes=(1, 0)), 0, axis)
    return v.ravel()


def snapshot(u, n, mass_ab, p, prefix, planes):
    """Planes of an x-fastest n^3 field plus global statistics."""
    s = np.abs(u).max()
    out = {prefix + "max": np.float64(s), prefix + "norm": np.float64(np.linalg.norm(u / s) * s)}
    Mu = mass_apply(u / s, (n, n, n), [(mass_ab, p)] * 3)
    out[prefix + "mass_norm"] = np.float64(np.sqrt(np.dot(u / s, Mu)) * s)
    t = u.reshape(n, n, n)  # [k][j][i]; copies, since u goes on changing in place
    if "z" in planes:
        out[prefix + "plane_z"] = t[n // 2].copy()
    if "y" in planes:
        out[prefix + "plane_y"] = t[:, n // 3, :].copy()
    return out


def run_case(L, name, p, E, dt, nsteps, seed, nthreads):
    import time

    sys.path.insert(0, os.path.join(ROOT, "iga-ads_gb300"))
    import ads_gb300 as ads
    from ads_gb300 import inputs

    L.ref_heat_steps_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp,
                                    ctypes.c_int]
    dims = [ads.Dimension(p, E) for _ in range(3)]
    u = inputs.initial_field(dims, seed=seed)
    n = E + p
    mass = tables(L, p, E)["mass"]
    out = dict(p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), nsteps=np.int32(nsteps), seed=np.int64(seed),
               threads=np.int32(nthreads), plane_z_index=np.int32(n // 2), plane_y_index=np.int32(n // 3))
    out["u0_norm"] = np.float64(np.linalg.norm(u))
    out["u0_sum"] = np.float64(u.sum())
    t0 = time.time()
    assert L.ref_heat_steps_mt(3, p, E, dt, 1, dp(u), nthreads) == 0
    out.update(snapshot(u, n, mass, p, "u1_", "z"))
    print(f"{name}: step 1 done in {time.time() - t0:.0f} s", flush=True)
    assert L.ref_heat_steps_mt(3, p, E, dt, nsteps - 1, dp(u), nthreads) == 0
    out.update(snapshot(u, n, mass, p, "uN_", "zy"))
    out["seconds"] = np.float64(time.time() - t0)
    print(f"{name}: {nsteps} steps done in {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, flush=True)


def norms_case(L, nd, p, E, seed):
    """The reference's normL2 / normH1 of a seeded spline and its errorL2 /
    errorH1 against prod sin(pi x_d), plus the norms of that function
    (basic_simulation_2d/3d's quadrature loops)."""
    L.ref_norms.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]
    size = (E + p) ** nd
    u = (2.0 * splitmix_uniform(seed, size) - 1.0)
    out = np.zeros(6)
    assert L.ref_norms(nd, p, E, dp(u), dp(out)) == 0
    return dict(ndim=np.int32(nd), p=np.int32(p), elements=np.int32(E), seed=np.int64(seed), u=u, normL2=out[0],
                normH1=out[1], errorL2=out[2], errorH1=out[3], f_normL2=out[4], f_normH1=out[5])


NORM_CASES = [(2, 2, 9, 21), (3, 2, 6, 22), (3, 4, 5, 23), (2, 3, 11, 24)]


def validation_case(L, p, E, dt, nsteps):
    """The reference's validation example (Dirichlet on every side, exact
    solution e^{-2 pi^2 t} sin(pi x) sin(pi y)) run for nsteps."""
    L.ref_validation.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp]
    u = np.zeros((E + p) ** 2)
    err = np.zeros(2)
    assert L.ref_validation(p, E, dt, nsteps, dp(u), dp(err)) == 0
    return dict(p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), nsteps=np.int32(nsteps), uN=u,
                errorL2_percent=err[0], errorH1_percent=err[1])


def heat2d_dirichlet_case(L, p, E, dt, nsteps):
    """The reference's heat_2d example (row x = 0 held at the load vector of
    sin(pi y), x.fix_left()) from its initial state through nsteps."""
    L.ref_heat2d_dirichlet.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp]
    u = np.zeros((E + p) ** 2)
    row = np.zeros(E + p)
    assert L.ref_heat2d_dirichlet(p, E, dt, nsteps, dp(u), dp(row)) == 0
    u1 = np.zeros_like(u)
    assert L.ref_heat2d_dirichlet(p, E, dt, 1, dp(u1), dp(row)) == 0
    return dict(p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), nsteps=np.int32(nsteps), u1=u1, uN=u, row=row)


def run_self_case(L, name, p, E, dt, seed, nthreads):
    """The first step of a full-size run once more, on another thread count
    of the executor (the scatter order, and so the rounding, differs): the
    reference's disagreement with itself at that size, recorded like the run
    (<name>_self.npz)."""
    import time

    sys.path.insert(0, os.path.join(ROOT, "iga-ads_gb300"))
    import ads_gb300 as ads
    from ads_gb300 import inputs

    L.ref_heat_steps_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp,
                                    ctypes.c_int]
    u = inputs.initial_field([ads.Dimension(p, E) for _ in range(3)], seed=seed)
    n = E + p
    mass = tables(L, p, E)["mass"]
    out = dict(p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), seed=np.int64(seed), threads=np.int32(nthreads),
               u0_norm=np.float64(np.linalg.norm(u)))
    t0 = time.time()
    assert L.ref_heat_steps_mt(3, p, E, dt, 1, dp(u), nthreads) == 0
    out.update(snapshot(u, n, mass, p, "u1_", "z"))
    out["seconds"] = np.float64(time.time() - t0)
    np.savez_compressed(os.path.join(HERE, name + "_self.npz"), **out)
    print(f"wrote {name}_self after {time.time() - t0:.0f} s", flush=True)


def main_runs(names, nthreads):
    L = load_ref()
    for name, p, E, dt, nsteps, seed in RUNS:
        if not names or name in names:
            run_case(L, name, p, E, dt, nsteps, seed, nthreads)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--runs":
        return main_runs(sys.argv[2:], os.cpu_count() or 1)
    if len(sys.argv) > 2 and sys.argv[1] == "--runs-self":
        # python make_golden.py --runs-self NAME THREADS
        L = load_ref()
        name, p, E, dt, nsteps, seed = next(r for r in RUNS if r[0] == sys.argv[2])
        return run_self_case(L, name, p, E, dt, seed, int(sys.argv[3]) if len(sys.argv) > 3 else 4)
    L = load_ref()
    for name, which, p, E, dt, seed in FORM_CASES:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **form_case(L, which, p, E, dt, seed))
        print("wrote", name)
    for nd, p, E, seed in NORM_CASES:
        np.savez_compressed(os.path.join(HERE, f"norms_{nd}d_p{p}_e{E}.npz"), **norms_case(L, nd, p, E, seed))
    np.savez_compressed(os.path.join(HERE, "validation_2d_p2_e16.npz"), **validation_case(L, 2, 16, 1e-4, 500))
    np.savez_compressed(os.path.join(HERE, "heat2d_dirichlet_p2_e32.npz"),
                        **heat2d_dirichlet_case(L, 2, 32, 1e-5, 100))
    for p, E in [(2, 8), (3, 7), (4, 12), (2, 32), (4, 36)]:
        np.savez_compressed(os.path.join(HERE, f"tables_p{p}_e{E}.npz"), **tables(L, p, E))
    np.savez_compressed(os.path.join(HERE, "solver_known_answers.npz"), **known_answers(L))
    for nd, p, E, dt, ns, seed, mode in CASES:
        name = f"heat_{nd}d_p{p}_e{E}" + ("_literal" if mode else "")
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **heat_case(L, nd, p, E, dt, ns, seed, mode))
        print("wrote", name)


if __name__ == "__main__":
    main()
