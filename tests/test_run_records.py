"""The full-size run records in tests/golden (made by the reference's own
code, make_golden.py --runs / --runs-self, and by the oracle, oracle_run.py)
against each other, on the CPU: they start from the field the package
recreates, and the CPU forms of the reference's algorithm disagree among
themselves by the amounts the full-size GPU checks take as their bound
(tests/test_gpu_fullsize.py)."""
from __future__ import annotations

import os

import numpy as np
import pytest

import ads_gb300 as ads
import oracle
from ads_gb300 import inputs
from conftest import GOLDEN

C3 = ("run_3d_p4_e256", "run_3d_p4_e256_self", "run_3d_p4_e256_oracle", "run_3d_p4_e256_oracle_seq")


def _load(name):
    path = os.path.join(GOLDEN, name + ".npz")
    assert os.path.exists(path), f"{name}.npz missing"
    return np.load(path)


def _apart(a, b, prefix):
    errs = [oracle.rel_l2(a[prefix + "plane_z"], b[prefix + "plane_z"])]
    if prefix + "plane_y" in a.files and prefix + "plane_y" in b.files:
        errs.append(oracle.rel_l2(a[prefix + "plane_y"], b[prefix + "plane_y"]))
    for k in ("norm", "mass_norm"):
        errs.append(abs(float(a[prefix + k]) - float(b[prefix + k])) / float(b[prefix + k]))
    return max(errs)


@pytest.mark.parametrize("name,p,E", [("run_3d_p2_e128", 2, 128), ("run_3d_p4_e256", 4, 256)])
def test_records_start_from_the_packages_field(name, p, E):
    g = _load(name)
    assert (int(g["p"]), int(g["elements"])) == (p, E)
    u0 = inputs.initial_field([ads.Dimension(p, E) for _ in range(3)], seed=int(g["seed"]))
    assert abs(np.linalg.norm(u0) - float(g["u0_norm"])) <= 1e-14 * float(g["u0_norm"])
    for other in (n for n in C3[1:] if n.startswith(name)):
        assert abs(float(_load(other)["u0_norm"]) - float(g["u0_norm"])) <= 1e-14 * float(g["u0_norm"])


def test_c3_cpu_forms_disagree_as_recorded():
    ref, ref4, orc, seq = (_load(n) for n in C3)
    # the reference's executor on 8 and 4 threads: the same scatter order up to
    # the chunking, a few ulp of the mass matrix's condition
    assert _apart(ref4, ref, "u1_") < 2e-13
    # the oracle's executor against the reference's
    assert _apart(orc, ref, "u1_") < 2e-12
    # the sequential element loop against both executors: the largest spread,
    # which the GPU's first-step bound doubles
    spread = max(_apart(seq, ref, "u1_"), _apart(seq, orc, "u1_"), _apart(seq, ref4, "u1_"))
    assert 1e-12 < spread < 5e-11
    # after 20 steps the growing top modes dominate and the runs agree closely
    assert _apart(orc, ref, "uN_") < 1e-13
