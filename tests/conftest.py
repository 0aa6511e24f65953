"""Shared test set-up: paths, the gpu marker and the build of the in-tree
libraries (the CUDA engine and the CPU oracle are both built here if stale)."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "iga-ads_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_sessionstart(session):
    import build as engine_build  # iga-ads_gb300/build.py

    engine_build.build()
    if os.environ.get("ADSG_LIBRARY") == "checked":  # the bounds-checked debug library
        engine_build.build(checked=True)
    import oracle

    oracle.build()


def pytest_sessionfinish(session, exitstatus):
    """Under the bounds-checked library, write what its kernels' checks
    caught to the file ADSG_BOUNDS_REPORT names (read by the test that runs
    the parity cases under the checks)."""
    path = os.environ.get("ADSG_BOUNDS_REPORT")
    if path and os.environ.get("ADSG_LIBRARY") == "checked" and gpu_available():
        import json

        import ads_gb300

        with open(path, "w") as f:
            json.dump(ads_gb300.debug_bounds(), f)


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not gpu_available():
        pytest.fail("this test needs a GPU (it is marked gpu)")
    import torch

    return torch.device("cuda:0")
