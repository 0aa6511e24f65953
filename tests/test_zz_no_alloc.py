"""adsg_heat_rhs_noalloc: the heat RHS for callers that cannot allocate device
memory (a host application that owns all device memory through its own pool,
or a loop that must not pay cudaMalloc's implicit synchronisation).  It must
give what adsg_heat_rhs gives, call after call, through the C-ABI.

This file is collected last on purpose: the entry point keeps a process-wide
device array, and the test must pass both alone in a fresh process and after
every other test."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import ads_gb300 as ads
import oracle

pytestmark = pytest.mark.gpu


def _noalloc():
    fn = ads.library().adsg_heat_rhs_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.POINTER(ads.DimDesc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                   ctypes.c_void_p]
    return fn


def _descs(dims):
    return (ads.DimDesc * len(dims))(*[d.descriptor() for d in dims])


@pytest.mark.parametrize("p,elements", [((2, 2, 2), (30, 24, 20)), ((4, 3), (60, 41)), ((3,), (100,))])
def test_noalloc_matches_context_rhs_on_consecutive_calls(p, elements, cuda):
    import torch

    dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
    ctx = ads.Context(dims)
    descs = _descs(dims)
    fn = _noalloc()
    rng = np.random.default_rng(sum(elements))
    for call, dt in enumerate((1e-5, 3e-4)):  # two calls in a row, different inputs and dt
        u = torch.from_numpy(rng.uniform(-1, 1, ctx.size)).to(cuda)
        ref = torch.empty_like(u)
        got = torch.full_like(u, float("nan"))
        ctx.heat_rhs(u, ref, dt)
        ctx.synchronize()
        torch.cuda.synchronize()
        code = fn(len(dims), descs, u.data_ptr(), got.data_ptr(), dt, None)
        assert code == 0, ads.library().adsg_last_error()
        torch.cuda.synchronize()
        assert oracle.rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-13, f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_array(cuda):
    import torch

    fn = _noalloc()
    big = [ads.Dimension(2, 98) for _ in range(3)]  # 100^3 dofs > 2^19
    u = torch.zeros(8, dtype=torch.float64, device=cuda)
    r = torch.zeros(8, dtype=torch.float64, device=cuda)
    assert fn(3, _descs(big), u.data_ptr(), r.data_ptr(), 1e-6, None) == -2
    assert b"ADSG_NOALLOC_MAX_DOFS" in ads.library().adsg_last_error()
    wide = [ads.Dimension(2, 1100)]  # 1102 dofs along x > 1024
    assert fn(1, _descs(wide), u.data_ptr(), r.data_ptr(), 1e-6, None) == -2
    assert b"ADSG_NOALLOC_MAX_N" in ads.library().adsg_last_error()


def test_noalloc_back_to_back_on_one_stream_allocates_nothing(cuda):
    """Several calls on one stream with no synchronisation between them, with
    different shapes and dt, each checked against the context's RHS; after a
    first call the device's free memory does not change over the calls, as
    the entry point allocates nothing."""
    import torch

    fn = _noalloc()
    cases = [((2, 2, 2), (30, 24, 20), 1e-5), ((4, 3), (60, 41), 3e-4), ((3,), (100,), 2e-3),
             ((2, 2, 2), (12, 40, 9), 7e-5), ((4, 4), (50, 50), 1e-6)]
    rng = np.random.default_rng(99)
    prepared = []
    for p, elements, dt in cases:
        dims = [ads.Dimension(pp, e) for pp, e in zip(p, elements)]
        ctx = ads.Context(dims)
        u = torch.from_numpy(rng.uniform(-1, 1, ctx.size)).to(cuda)
        ref = torch.empty_like(u)
        ctx.heat_rhs(u, ref, dt)
        ctx.synchronize()
        prepared.append((dims, _descs(dims), u, ref, torch.full_like(u, float("nan")), dt, ctx))
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    dims, descs, u, ref, got, dt, _ = prepared[0]
    assert fn(len(dims), descs, u.data_ptr(), got.data_ptr(), dt, ctypes.c_void_p(stream.cuda_stream)) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for dims, descs, u, ref, got, dt, _ in prepared:
            code = fn(len(dims), descs, u.data_ptr(), got.data_ptr(), dt, ctypes.c_void_p(stream.cuda_stream))
            assert code == 0, ads.library().adsg_last_error()
    stream.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    for k, (dims, descs, u, ref, got, dt, _) in enumerate(prepared):
        assert oracle.rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-13, f"case {k}"
