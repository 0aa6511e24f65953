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
    import oracle

    oracle.build()


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
