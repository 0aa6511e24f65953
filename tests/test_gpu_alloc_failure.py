"""Device allocation failures, made on the host: the library's hook
(adsg_test_fail_device_alloc) fails its k-th device allocation from now on
as cudaMalloc does on a full device.  For k = 0, 1, 2, ... a context, a batch
and an adjoint are created under a failure of their k-th allocation until
they need fewer than k + 1; every creation that meets the failure must
return ADSG_ERR_NOMEM ("out of memory") and free what it had taken, and
where the library absorbs a failure (the launch-mode tuner's work buffer:
the context then keeps plain launches) the object must still compute the
right steps.  No GPU fault is involved: nothing reaches the device that a
full device would not also see."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import ads_gb300 as ads
import oracle
from _tol import STEP, check

pytestmark = pytest.mark.gpu

NOMEM = 1002


def _free_bytes():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _under_each_failure(make, limit=400):
    """Calls make() with its k-th device allocation failing, k = 0, 1, ...:
    returns (creations that reported the failure, objects that absorbed it,
    the object made once k passed its last allocation)."""
    failed, absorbed = 0, []
    for k in range(limit):
        ads.test_fail_device_alloc(k)
        try:
            obj = make()
        except ads.AdsError as e:
            ads.test_fail_device_alloc(-1)
            assert e.code == NOMEM, str(e)
            assert "out of memory" in str(e), str(e)
            failed += 1
            continue
        if ads.test_fail_device_alloc(-1) >= 0:  # fewer than k + 1 allocations: all were failed in turn
            return failed, absorbed, obj
        absorbed.append(obj)
    raise AssertionError(f"more than {limit} device allocations")


def test_context_creation_under_each_allocation_failure(cuda):
    """130^3 dofs, so that a leaked work tensor (17.6 MB) would show in the
    device's free memory."""
    dims = [ads.Dimension(2, 128) for _ in range(3)]
    ref_ctx = ads.Context(dims)  # also fills the process's tuning caches
    u0 = np.random.default_rng(5).uniform(-1, 1, ref_ctx.size)
    ref = u0.copy()
    ref_ctx.heat_steps_host(ref, 1e-6, 2)
    free0 = _free_bytes()
    failed, absorbed, ctx = _under_each_failure(lambda: ads.Context(dims))
    print(f"[alloc] context: {failed} creations reported the failure, {len(absorbed)} absorbed it")
    assert failed >= 30  # per direction its tables, then the work tensors and the state
    assert len(absorbed) == 1 and not absorbed[0].launch_pdl() and not absorbed[0].step_graphs()
    for c in absorbed + [ctx]:
        u = u0.copy()
        c.heat_steps_host(u, 1e-6, 2)
        check("130^3 context made through an allocation failure, 2 steps", oracle.rel_l2(u, ref), 2 * STEP)
        c.close()
    leaked = free0 - _free_bytes()
    assert leaked < 8 << 20, f"{leaked} bytes of device memory not returned"
    ref_ctx.close()


def test_batch_creation_under_each_allocation_failure(cuda):
    specs = [(2, 2, 40, 1e-5), (3, 3, 12, 1e-6), (3, 2, 20, 1e-6)]
    u0 = [np.random.default_rng(10 + i).uniform(-1, 1, (e + p) ** nd) for i, (nd, p, e, _) in enumerate(specs)]
    failed, absorbed, b = _under_each_failure(lambda: ads.Batch(specs))
    print(f"[alloc] batch: {failed} creations reported the failure, {len(absorbed)} absorbed it")
    assert failed >= 10
    for bb in absorbed + [b]:
        for i, u in enumerate(u0):
            bb.set_state(i, u)
        bb.steps(2)
        bb.synchronize()
        for i, (nd, p, e, dt) in enumerate(specs):
            ref = oracle.Problem([p] * nd, [e] * nd).heat_steps(u0[i], dt, 2)
            check(f"batch instance {i} made through an allocation failure", oracle.rel_l2(bb.get_state(i), ref),
                  2 * STEP)
        bb.close()


def test_adjoint_and_gauss_point_space_under_each_allocation_failure(cuda):
    dims = [ads.Dimension(2, 10), ads.Dimension(2, 12), ads.Dimension(2, 9)]
    ctx = ads.Context(dims)
    failed, absorbed, adj = _under_each_failure(lambda: ads.Adjoint(ctx, 6, 1e-6))
    # one failure is absorbed: kappa at the Gauss points, without which the
    # passes interpolate the coefficients (the same gradients, bit for bit)
    assert failed >= 5 and len(absorbed) == 1
    u0 = torch.from_numpy(np.random.default_rng(8).uniform(-1, 1, ctx.size)).cuda()
    kap = torch.from_numpy(1.0 + 0.3 * np.random.default_rng(9).uniform(-1, 1, ctx.size)).cuda()
    res = []
    for a in (adj, absorbed[0]):
        uT, gu, gk = torch.empty_like(u0), torch.empty_like(u0), torch.empty_like(u0)
        a.forward(u0, kap, uT)
        a.backward(uT, gu, gk)
        ctx.synchronize()
        res.append((uT.clone(), gu.clone(), gk.clone()))
        a.close()
    for x, y in zip(*res):
        assert torch.equal(x, y)
    # the Gauss-point work space, taken on first use
    E, q = (10, 12, 9), 3
    u = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, ctx.size)).cuda()
    val = torch.empty(int(np.prod(E)) * q ** 3, dtype=torch.float64, device="cuda")
    ads.test_fail_device_alloc(0)
    with pytest.raises(ads.AdsError) as err:
        ctx.eval_quad(u, val)
    ads.test_fail_device_alloc(-1)
    assert err.value.code == NOMEM
    ctx.eval_quad(u, val)  # the next call takes the space and works
    ctx.synchronize()
    assert torch.isfinite(val).all()
    ctx.close()
