"""C++ host code drops in: (1) a program built against the reference's own
classes (ads::simulation_3d, ads::dimension, lin::tensor) compiles against
ads/gpu.hpp -- built where the reference sources exist; (2) a program over
stand-ins of the reference's types with exactly the members ads/gpu.hpp
reads runs the bridge's compute_rhs_heat, solve and heat_steps on the GPU
against the oracle; (3) a standalone C++ program over the C-ABI reproduces
the reference test's 3D known-answer ADS system on the GPU."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def _have_reference() -> bool:
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "have-ref"], capture_output=True, text=True)
    return r.stdout.strip() == "yes"


@pytest.mark.skipif(not _have_reference(), reason="reference sources not present on this machine")
def test_reference_program_builds_against_the_bridge():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    exe = os.path.join(ROOT, "oracle", "_ref", "dropin")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith(("no-gpu", "ok")), out.stdout


def _build_standalone(tmp_path):
    exe = str(tmp_path / "capi_known_answers")
    lib_dir = os.path.join(ROOT, "iga-ads_gb300", "ads_gb300")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "iga-ads_gb300", "include"), "-I",
           os.path.join(ROOT, "include"), "-o", exe, os.path.join(ROOT, "tests", "cpp", "capi_known_answers.cpp"),
           os.path.join(lib_dir, "libads_gb300.so"), f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_standalone_program_compiles(tmp_path):
    _build_standalone(tmp_path)


@pytest.mark.gpu
def test_standalone_program_known_answers_on_gpu(tmp_path, cuda):
    exe = _build_standalone(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr


def _build_bridge(tmp_path):
    import oracle

    oracle.build()
    exe = str(tmp_path / "bridge_gpu")
    lib_dir = os.path.join(ROOT, "iga-ads_gb300", "ads_gb300")
    orc_dir = os.path.join(ROOT, "oracle", "_build")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    cuda_lib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                 os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                                 os.path.join(cuda, "targets", "x86_64-linux", "lib"))
                     if os.path.exists(os.path.join(d, "libcudart.so"))), os.path.join(cuda, "lib64"))
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "iga-ads_gb300", "include"), "-I",
           os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"), "-I", os.path.join(cuda, "include"),
           "-o", exe, os.path.join(ROOT, "tests", "cpp", "bridge_gpu.cpp"), os.path.join(lib_dir, "libads_gb300.so"),
           os.path.join(orc_dir, "libads_oracle.so"), "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{lib_dir}",
           f"-Wl,-rpath,{orc_dir}", f"-Wl,-rpath,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_bridge_program_compiles(tmp_path):
    _build_bridge(tmp_path)


@pytest.mark.gpu
def test_bridge_on_gpu_against_oracle(tmp_path, cuda):
    """ads::gpu::context built from reference-shaped dimensions runs
    compute_rhs_heat, solve and heat_steps on the GPU; each matches the
    oracle.  ads::gpu::adjoint (the C++ reverse-mode class) passes the
    dot-product identity and central differences of the mass-norm loss (the
    program prints every error and its bound)."""
    exe = _build_bridge(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout + out.stderr
