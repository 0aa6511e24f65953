"""The C-ABI library loads and exports every entry point include/*.h declares;
argument checks answer with LAPACK-style negative codes before touching the
GPU.  CPU only: no device call is made."""
from __future__ import annotations

import ctypes
import glob
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import ads_gb300 as ads
from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(adsg_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("adsg_ctx_create", "adsg_heat_rhs", "adsg_ads_solve", "adsg_heat_steps", "adsg_dgbtrs_"):
        assert must in names


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(name):
    lib = ads.library()
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_exported_symbols_are_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", ads.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (adsg_\w+)", out))
    assert set(declared_functions()) <= exported


def _dgbtrs(trans=b"N", n=4, kl=1, ku=1, nrhs=1, ldab=4, ldb=4, ab=None, ipiv=None, b=None):
    lib = ads.library()
    ab = np.zeros(max(ldab, 1) * max(n, 1)) if ab is None else ab
    ipiv = np.arange(1, max(n, 1) + 1, dtype=np.int32) if ipiv is None else ipiv
    b = np.zeros(max(ldb, 1) * max(nrhs, 1)) if b is None else b
    ints = [ctypes.c_int(v) for v in (n, kl, ku, nrhs, ldab, ldb)]
    info = ctypes.c_int(99)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    code = lib.adsg_dgbtrs_(trans, ctypes.byref(ints[0]), ctypes.byref(ints[1]), ctypes.byref(ints[2]),
                            ctypes.byref(ints[3]), ab.ctypes.data_as(dp), ctypes.byref(ints[4]),
                            ipiv.ctypes.data_as(ip), b.ctypes.data_as(dp), ctypes.byref(ints[5]), ctypes.byref(info))
    return code, info.value


@pytest.mark.parametrize("kw,code", [
    (dict(trans=b"X"), -1),
    (dict(n=-1), -2),
    (dict(kl=-1), -3),
    (dict(ku=-1), -4),
    (dict(nrhs=-1), -5),
    (dict(ldab=2), -7),
    (dict(ldb=2), -10),
])
def test_dgbtrs_argument_errors_match_lapack(kw, code):
    c, info = _dgbtrs(**kw)
    assert c == code and info == code


def test_dgbtrs_empty_problem_is_a_no_op():
    assert _dgbtrs(n=0, ldb=1) == (0, 0)
    assert _dgbtrs(nrhs=0) == (0, 0)


def test_dgbtrs_unsolved_cases_report_positive_info_without_gpu():
    """A caller that reads only info sees every case where b is left
    unsolved: a band beyond the supported width (info = n + 1) and an exactly
    zero U diagonal (info = its 1-based column).  Both are decided before any
    device call."""
    n, kl, ku = 40, 17, 17
    ldab = 2 * kl + ku + 1
    ab = np.ones(ldab * n)
    b = np.arange(float(n))
    code, info = _dgbtrs(n=n, kl=kl, ku=ku, nrhs=1, ldab=ldab, ldb=n, ab=ab, b=b)
    assert code == 1005 and info == n + 1
    np.testing.assert_array_equal(b, np.arange(float(n)))
    n, kl, ku = 6, 1, 1
    ldab = 4
    ab = np.ones(ldab * n)
    ab[3 * ldab + kl + ku] = 0.0  # U(4, 4) = 0
    code, info = _dgbtrs(n=n, kl=kl, ku=ku, nrhs=1, ldab=ldab, ldb=n, ab=ab, b=np.ones(n))
    assert code == 1003 and info == 4


def test_dgbtrs_checked_aborts_where_info_would_be_ignored():
    """The entry for callers that never read info (the reference's own
    band_solve.hpp) stops the process with the reason instead of returning
    an unsolved b.  Run in a child process; the failing case is rejected on
    the host, before any device call."""
    code = (
        "import ctypes, numpy as np, sys; sys.path.insert(0, %r); import ads_gb300 as a\n"
        "lib = a.library(); n, kl, ku = 40, 17, 17; ldab = 2*kl+ku+1\n"
        "ab = np.ones(ldab*n); b = np.zeros(n); piv = np.arange(1, n+1, dtype=np.int32)\n"
        "I = [ctypes.c_int(v) for v in (n, kl, ku, 1, ldab, n)]; info = ctypes.c_int(0)\n"
        "dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)\n"
        "lib.adsg_dgbtrs_checked_(b'N', *[ctypes.byref(I[k]) for k in range(4)], ab.ctypes.data_as(dp),\n"
        "    ctypes.byref(I[4]), piv.ctypes.data_as(ip), b.ctypes.data_as(dp), ctypes.byref(I[5]), ctypes.byref(info))\n"
        "print('returned')\n" % os.path.join(ROOT, "iga-ads_gb300"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "returned" not in r.stdout
    assert "aborting" in r.stderr and "band wider" in r.stderr


def test_ctx_create_rejects_bad_arguments_without_gpu():
    lib = ads.library()
    h = ctypes.c_void_p()
    assert lib.adsg_ctx_create(0, None, ctypes.byref(h)) == -1
    assert lib.adsg_ctx_create(4, None, ctypes.byref(h)) == -1
    assert lib.adsg_ctx_create(2, None, ctypes.byref(h)) == -2
    bad = (ads.DimDesc * 1)()
    assert lib.adsg_ctx_create(1, bad, ctypes.byref(h)) == -2
    assert b"invalid" in lib.adsg_last_error()


def test_ctx_create_rejects_tensors_beyond_int32_indexing_without_gpu():
    """1300^3 dofs (> 2^31) is refused with -2 before any device call."""
    lib = ads.library()
    d = ads.Dimension(2, 1298)
    descs = (ads.DimDesc * 3)(d._desc, d._desc, d._desc)
    h = ctypes.c_void_p()
    assert lib.adsg_ctx_create(3, descs, ctypes.byref(h)) == -2
    assert b"2^31" in lib.adsg_last_error() and not h.value


def test_device_entry_points_reject_null_context():
    lib = ads.library()
    assert lib.adsg_heat_rhs(None, None, None, 1.0) == -1
    assert lib.adsg_ads_solve(None, None, None) == -1
    assert lib.adsg_heat_steps(None, None, 1.0, 1) == -1
    assert lib.adsg_ctx_destroy(None) == 0


def test_every_engine_source_is_built():
    """iga-ads_gb300/build.py lists every CUDA and C++ source of the engine
    (a source left out would silently drop its entry points)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("engine_build", os.path.join(ROOT, "iga-ads_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    csrc = os.path.join(ROOT, "iga-ads_gb300", "csrc")
    on_disk = sorted(f for f in os.listdir(csrc) if f.endswith((".cu", ".cpp")))
    assert sorted(b.CUDA_SOURCES + b.CXX_SOURCES) == on_disk
