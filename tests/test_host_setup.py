"""The engine's host-side set-up (adsg_dim_create: basis tables, mass and
stiffness bands, pivoted band LU) against the reference's own tables in the
golden fixtures.  Runs on the CPU: no GPU call is made."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

import ads_gb300 as ads
from conftest import GOLDEN

TABLES = sorted(glob.glob(os.path.join(GOLDEN, "tables_*.npz")))


@pytest.mark.parametrize("path", TABLES, ids=os.path.basename)
def test_dimension_tables_match_reference(path):
    g = np.load(path)
    p, E = int(g["p"]), int(g["elements"])
    d = ads.Dimension(p, E)
    assert d.dofs() == E + p
    t = d.tables()
    np.testing.assert_array_equal(t["btab"], g["btab"])
    np.testing.assert_array_equal(t["w"], g["w"])
    np.testing.assert_array_equal(t["J"], g["J"])
    np.testing.assert_array_equal(t["first_dofs"], g["first_dofs"])
    np.testing.assert_array_equal(d.form_band(0).ravel(), g["mass"])
    np.testing.assert_array_equal(d.form_band(1).ravel(), g["stiffness"])
    np.testing.assert_array_equal(t["ipiv"], g["ipiv"])
    scale = np.abs(g["lu"]).max()
    assert np.abs(t["lu"] - g["lu"]).max() <= 8 * np.finfo(float).eps * scale
    assert (t["kl"], t["ku"], t["ldab"]) == (p, p, 3 * p + 1)


def test_fix_dof_identity_row():
    d = ads.Dimension(2, 6)
    d.fix_left()
    M = d.form_band(0)  # row k=0: only the diagonal, equal to 1
    kl = ku = 2
    assert M[0, kl + ku] == 1.0
    for j in (1, 2):
        assert M[j, kl + ku - j] == 0.0
    t = d.tables()
    assert t["lu"][kl + ku] == 1.0  # U(0,0) of the refactorised band


@pytest.mark.parametrize("args,code", [
    ((0, 4), -1), ((9, 4), -1), ((2, 0), -2),
])
def test_dimension_rejects_bad_arguments(args, code):
    with pytest.raises(ads.AdsError) as ei:
        ads.Dimension(*args)
    assert ei.value.code == code


def test_dimension_rejects_empty_interval():
    with pytest.raises(ads.AdsError) as ei:
        ads.Dimension(2, 4, 1.0, 1.0)
    assert ei.value.code == -4


def test_initial_field_is_seeded_and_smooth_plus_noise():
    from ads_gb300 import inputs

    dims = [ads.Dimension(2, 8) for _ in range(3)]
    a = inputs.initial_field(dims, seed=5)
    b = inputs.initial_field(dims, seed=5)
    c = inputs.initial_field(dims, seed=6)
    np.testing.assert_array_equal(a, b)
    assert np.abs(a - c).max() > 0
    assert np.abs(a - c).max() <= 2e-2 + 1e-15
    assert a.size == 10 ** 3
    u = inputs.splitmix_uniform(7, 100000)
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01


def test_direction_tables_on_the_host(tmp_path):
    """tests/cpp/tables_check.cpp, built from the engine's host sources alone:
    LAPACK-order solve tables, the symmetric row range of the pair-sum passes,
    the two-ended factorisation (built exactly for n >= 4k+2, self-checked
    against the LAPACK-order solve) and its row-scaled form, degrees 1-4."""
    import shutil
    import subprocess

    from conftest import ROOT

    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    csrc = os.path.join(ROOT, "iga-ads_gb300", "csrc")
    exe = str(tmp_path / "tables_check")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", csrc, "-I", cuda_inc, "-o", exe,
           os.path.join(ROOT, "tests", "cpp", "tables_check.cpp"), os.path.join(csrc, "adsg_tables.cpp"),
           os.path.join(csrc, "adsg_host.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout[-2000:]
