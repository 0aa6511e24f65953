"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer (the
reference's own CI runs its suite that way: cmake/Sanitizers.cmake, ASan and
UBSan).  Two programs, built with -fsanitize=address,undefined and no
recovery, so that any out-of-bounds access, leak, use after free, signed
overflow or misaligned load ends the run with a report:

- tests/cpp/tables_check.cpp with the engine's host sources (adsg_host.cpp:
  basis tables, Gauss rules, mass bands and their banded LU; adsg_tables.cpp:
  row bands, solve tables, the two-ended factorisation and its row-scaled
  form), degrees 1-4;
- tests/cpp/oracle_check.c with the CPU oracle (oracle/ads_oracle.c): every
  entry the tests call on 1D/2D/3D grids of degree 1-4, threaded and
  sequential."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from conftest import ROOT

FLAGS = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g", "-O1"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")


def _sanitizers_available(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text("int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", *FLAGS, "-o", str(tmp_path / "probe"), str(src)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("the compiler has no ASan/UBSan runtime here: " + r.stderr.strip()[-200:])


def _run(cmd, exe):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=ENV)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), (out.stdout[-2000:], out.stderr[-4000:])
    assert "runtime error" not in out.stderr, out.stderr[-4000:]


def test_engine_host_sources_under_sanitizers(tmp_path):
    _sanitizers_available(tmp_path)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    csrc = os.path.join(ROOT, "iga-ads_gb300", "csrc")
    exe = str(tmp_path / "tables_check_san")
    _run(["g++", "-std=c++17", *FLAGS, "-I", os.path.join(ROOT, "include"), "-I", csrc, "-I", cuda_inc, "-o", exe,
          os.path.join(ROOT, "tests", "cpp", "tables_check.cpp"), os.path.join(csrc, "adsg_tables.cpp"),
          os.path.join(csrc, "adsg_host.cpp")], exe)


def test_oracle_under_sanitizers(tmp_path):
    _sanitizers_available(tmp_path)
    exe = str(tmp_path / "oracle_check_san")
    _run(["gcc", "-std=c11", *FLAGS, "-ffp-contract=off", "-I", os.path.join(ROOT, "oracle"), "-o", exe,
          os.path.join(ROOT, "tests", "cpp", "oracle_check.c"), os.path.join(ROOT, "oracle", "ads_oracle.c"),
          "-lpthread", "-lm"], exe)
