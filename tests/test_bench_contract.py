"""bench.py's host-side pieces, on the CPU: the workload descriptions, the
DRAM-traffic figures from ncu, the clock-record parser and the reference
arm's JSON line (the CPU oracle on a small grid, with the same warm-up, step
count, initial field and config as our arm)."""
from __future__ import annotations

import importlib.util
import json
import os
import types

import pytest

from conftest import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["heat2d_p2_32", "heat3d_p2_128", "heat3d_p4_256", "adjoint_p2_96"])
def test_workload_descriptions(name):
    b = _bench()
    nd, p, E, dt = b.WORKLOADS[name]
    cfg = b.workload_config(name)
    assert cfg["dofs"] == (E + p) ** nd
    assert (cfg["ndim"], cfg["p"], cfg["elements"], cfg["dt"]) == (nd, p, E, dt)
    assert f"{E}^{nd} elements" in cfg["workload"] and f"{p + 1}-point Gauss" in cfg["workload"]


def test_profiled_traffic_rows():
    """Every stage of the two 3D workloads has a measured row; a workload
    without rows of its own takes the larger-than-L2 p=4 rows."""
    b = _bench()
    stages = ("rhs_outer", "rhs_middle", "rhs_x", "solve_x", "solve_y", "solve_z")
    for w in ("heat3d_p2_128", "heat3d_p4_256"):
        per = [b.profiled_traffic(s, 1, w) for s in stages]
        assert all(v is not None and 0 < v < 64 for v in per), (w, per)
    own = [b.profiled_traffic(s, 1, "heat3d_p4_256") for s in stages]
    assert [b.profiled_traffic(s, 1, "heat2d_p2_32") for s in stages] == own
    assert b.profiled_traffic("rhs_middle", 1000, "heat3d_p2_128") == pytest.approx(
        1000 * b.profiled_traffic("rhs_middle", 1, "heat3d_p2_128"))
    assert b.profiled_traffic("no_such_stage", 1, "heat3d_p2_128") is None


class _FakeSmi:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def test_clock_record_parser():
    """The clocks line of the bench: median SM clock under load, maximum
    clock, and every throttle reason seen Active in any sample."""
    b = _bench()
    s = b.ClockSampler(0)
    s.proc = _FakeSmi()
    s.lines = [
        "2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "2040, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
        "2070, 2070, 1390.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    rec = s.stop()
    assert rec == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    s2 = b.ClockSampler(0)
    s2.proc = _FakeSmi()
    s2.lines = ["1200, 2070, 700, 0x8, Active, Not Active, Active, Not Active"]
    rec2 = s2.stop()
    assert rec2["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"] and rec2["sm_mhz"] == 1200.0
    assert b.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


def test_reference_arm_line(capsys):
    """--impl reference on the 2D workload: the CPU oracle's step, one JSON
    line carrying impl, cpu_baseline (kind, cores, sample) and an e2e block
    with no host-device traffic, on the same metric as our arm."""
    b = _bench()
    args = types.SimpleNamespace(gpus=1, steps=2, warmup=1, impl="reference", workload="heat2d_p2_32",
                                 no_cpu_baseline=False)
    assert b.run_reference(args, b.workload_config("heat2d_p2_32")) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == b.METRIC and line["unit"] == "DOF-updates/s"
    assert line["higher_is_better"] is True and line["steps"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "DOF-updates/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["dofs"] == 34 * 34
    assert line["warmup"] == 1 and line["data"] == b.DATA
    assert line["config"] == b.workload_config("heat2d_p2_32")


def test_reference_arm_initial_field_matches_ours():
    """The reference arm builds the initial field from the oracle's tables
    (bit-identical to the reference's); it equals the engine's host-side
    field to rounding."""
    import numpy as np

    import ads_gb300 as ads
    import oracle
    from ads_gb300 import inputs

    b = _bench()
    pr = oracle.Problem([2, 2], [32, 32])
    mine = inputs.initial_field([b._OracleDim(pr, d) for d in range(2)], seed=0)
    ours = inputs.initial_field([ads.Dimension(2, 32) for _ in range(2)], seed=0)
    assert np.abs(mine - ours).max() <= 1e-15
