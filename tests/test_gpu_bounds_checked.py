"""The parity cases under device-side bounds checks: the debug library
(libads_gb300_checked.so, -DADSG_BOUNDS_CHECK=1) compares every global index
of the step, solve, batch, element and Gauss-point kernels with its buffer's
extent and every shared-memory tile with the launch's shared memory,
skipping (never trapping on) a violation and counting it.  The small parity
cases of the GPU suite run against that library in a child process, which
reports the count at the end; it must pass and count nothing.  This stands in
for a memory checker, which is closed on this machine."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

FILES = ["tests/test_gpu_parity.py", "tests/test_gpu_batch.py", "tests/test_gpu_quad.py", "tests/test_gpu_forms.py",
         "tests/test_gpu_general.py", "tests/test_gpu_robustness.py", "tests/test_gpu_adjoint.py"]


def test_release_build_has_no_bounds_records():
    import ads_gb300 as ads

    if os.environ.get("ADSG_LIBRARY") == "checked":
        pytest.skip("running under the checked library")
    with pytest.raises(ads.AdsError, match="bounds-checked"):
        ads.debug_bounds()


def test_parity_cases_under_device_bounds_checks(cuda, tmp_path):
    if os.environ.get("ADSG_LIBRARY") == "checked":
        pytest.skip("already running under the checked library")
    sys.path.insert(0, os.path.join(ROOT, "iga-ads_gb300"))
    import build as engine_build

    engine_build.build(checked=True)
    report = tmp_path / "bounds.json"
    env = dict(os.environ, ADSG_LIBRARY="checked", ADSG_BOUNDS_REPORT=str(report))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider", *FILES,
                        "-k", "not mixed_64 and not wait_runs_out"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    tail = (r.stdout + r.stderr)[-3000:]
    assert r.returncode == 0, tail
    rec = json.loads(report.read_text())
    print(f"[bounds] {rec} after: {r.stdout.strip().splitlines()[-1]}")
    assert rec["violations"] == 0, rec
