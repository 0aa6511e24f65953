"""Builds libads_gb300.so (the sm_103a engine and its C-ABI) in-tree.

Usage: python iga-ads_gb300/build.py [--force] [--checked]

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked with a
static CUDA runtime into ads_gb300/libads_gb300.so next to the Python package.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "ads_gb300", "libads_gb300.so")
# the debug build with device-side bounds checks (-DADSG_BOUNDS_CHECK=1)
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(HERE, "ads_gb300", "libads_gb300_checked.so")

CUDA_SOURCES = ["adsg_kernels.cu", "adsg_elem.cu", "adsg_capi.cu", "adsg_adjoint.cu", "adsg_points.cu", "adsg_general.cu",
                "adsg_batch.cu", "adsg_noalloc.cu", "adsg_quad.cu"]
CXX_SOURCES = ["adsg_host.cpp", "adsg_tables.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ads_gb300")


def _sources():
    return [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))], CXX_SOURCES


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    """Compile and link the engine; checked=True builds the bounds-checked
    debug library instead (its own objects, libads_gb300_checked.so)."""
    build_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    defs = ["-DADSG_BOUNDS_CHECK=1"] if checked else []
    os.makedirs(build_dir, exist_ok=True)
    cu, cxx = _sources()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "ads_gb300.h"))
    objs, jobs = [], []
    nv = nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    for s in cu:
        src = os.path.join(CSRC, s)
        obj = os.path.join(build_dir, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", *defs, *inc, "-c", src, "-o", obj])
    for s in cxx:
        src = os.path.join(CSRC, s)
        obj = os.path.join(build_dir, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nv, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", *defs, *inc, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_compile, jobs))
    if force or jobs or _stale(lib, objs):
        _compile([nv, *ARCH, "-shared", "-cudart", "static", "-Xlinker", f"-soname={os.path.basename(lib)}", "-o", lib,
                  *objs])
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--checked", action="store_true", help="the bounds-checked debug library")
    a = ap.parse_args()
    try:
        build(force=a.force, verbose=True, checked=a.checked)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
