"""The batched engine (one persistent cooperative launch for many uneven
instances) against the CPU oracle and against the plain per-instance path."""
from __future__ import annotations

import numpy as np
import pytest

import ads_gb300 as ads
import oracle
from _tol import STEP, check, oracle_self

pytestmark = pytest.mark.gpu

SMALL = [(2, 2, 17, 1e-5), (3, 4, 7, 1e-6), (2, 4, 40, 2e-6), (3, 2, 12, 1e-6), (3, 3, 9, 1e-6), (2, 3, 5, 1e-4),
         (3, 1, 6, 1e-5), (2, 1, 33, 1e-5)]


def test_batch_against_oracle_and_loop(cuda):
    b = ads.Batch(SMALL)
    rng = np.random.default_rng(7)
    u0 = [rng.uniform(-1, 1, n) for n in b.sizes]
    for i, u in enumerate(u0):
        b.set_state(i, u)
    b.steps(3)
    b.synchronize()
    got = [b.get_state(i) for i in range(len(SMALL))]
    selfd = []
    for i, (nd, p, e, dt) in enumerate(SMALL):
        pr = oracle.Problem([p] * nd, [e] * nd)
        selfd.append(oracle_self(pr, u0[i], dt, 3))
        check(f"batch {SMALL[i]} 3 steps", oracle.rel_l2(got[i], pr.heat_steps(u0[i], dt, 3)), 3 * STEP, selfd[i])
    # the same three steps through the plain per-instance kernels (their
    # autotuned solves may use the two-ended sweep, which rounds differently
    # from the batched kernel's LAPACK-order sweep)
    for i, u in enumerate(u0):
        b.set_state(i, u)
    b.steps_looped(3)
    b.synchronize()
    for i, (nd, p, e, dt) in enumerate(SMALL):
        check(f"batch vs looped {SMALL[i]}", oracle.rel_l2(b.get_state(i), got[i]), 3 * STEP, selfd[i])


@pytest.mark.parametrize("engine", ["0", "1"])
def test_batch_repeated_calls_and_parity(engine, cuda, monkeypatch):
    """Both engines (persistent kernel, concurrent per-instance graph) over
    repeated calls with odd and even step counts."""
    monkeypatch.setenv("ADSG_BATCH_ENGINE", engine)
    b = ads.Batch(SMALL[:4])
    rng = np.random.default_rng(8)
    u0 = [rng.uniform(-1, 1, n) for n in b.sizes]
    for i, u in enumerate(u0):
        b.set_state(i, u)
    for n in (1, 2, 1, 3):  # odd counts flip the state buffer, graphs are re-captured
        b.steps(n)
    b.synchronize()
    for i, (nd, p, e, dt) in enumerate(SMALL[:4]):
        pr = oracle.Problem([p] * nd, [e] * nd)
        check(f"batch engine {engine} {SMALL[i]} 7 steps", oracle.rel_l2(b.get_state(i), pr.heat_steps(u0[i], dt, 7)),
              7 * STEP, oracle_self(pr, u0[i], dt, 7))
    t = b.tuning()
    assert t["blocks_per_sm"] >= 1
    assert t["engine"] == ("concurrent" if engine == "1" else "persistent")


def test_mixed_64_batch_matches_plain_kernels(cuda):
    specs = ads.batch_specs(seed=0)
    assert len(specs) == 64 and sum(s[0] == 2 for s in specs) == 32
    b = ads.Batch(specs)
    rng = np.random.default_rng(9)
    u0 = [rng.uniform(-1e-2, 1e-2, n) for n in b.sizes]
    for i, u in enumerate(u0):
        b.set_state(i, u)
    b.steps(2)
    b.synchronize()
    got = [b.get_state(i) for i in range(64)]
    for i, u in enumerate(u0):
        b.set_state(i, u)
    b.steps_looped(2)
    b.synchronize()
    # the per-instance contexts may solve with the two-ended sweep, which
    # rounds differently from the batched kernel's LAPACK-order sweep; the
    # bound is the oracle's own spread at that instance's shape
    for i, (nd, p, e, dt) in enumerate(specs):
        err = oracle.rel_l2(b.get_state(i), got[i])
        if err > 2 * STEP:
            pr = oracle.Problem([p] * nd, [e] * nd)
            check(f"mixed-64 batch vs looped {specs[i]}", err, 2 * STEP, oracle_self(pr, u0[i], dt, 2))


def test_item_order_does_not_change_results(cuda, monkeypatch):
    """The persistent kernel hands out the same items in either order
    (stage-major, or a wavefront over groups of instances that fit in L2
    together): bitwise equal states on the seeded 64-instance set."""
    monkeypatch.setenv("ADSG_BATCH_ENGINE", "0")
    specs = ads.batch_specs(seed=0)
    rng = np.random.default_rng(4)
    out = []
    for order in ("0", "1"):
        monkeypatch.setenv("ADSG_BATCH_ORDER", order)
        b = ads.Batch(specs)
        assert b.tuning()["order"] == ("wavefront" if order == "1" else "stage-major")
        for i, n in enumerate(b.sizes):
            b.set_state(i, np.random.default_rng(100 + i).uniform(-1, 1, n))
        b.steps(3)
        b.synchronize()
        out.append([b.get_state(i) for i in range(len(specs))])
        b.close()
    for i in range(len(specs)):
        np.testing.assert_array_equal(out[0][i], out[1][i])


def test_batch_rejects_bad_specs():
    with pytest.raises(ads.AdsError):
        ads.Batch([(4, 2, 8, 1e-6)])
    with pytest.raises(ads.AdsError):
        ads.Batch([(3, 5, 8, 1e-6)])


def test_persistent_kernel_wait_runs_out_and_the_batch_recovers(cuda, monkeypatch):
    """Failure detection without a fault: every wait of the persistent kernel
    for an instance's previous stage is told to expect one work item more
    than exists, with a spin limit of a few thousand polls, so every wait runs
    out; each waiting block sets the error word and returns.
    adsg_batch_synchronize reports ADSG_ERR_DEVICE (and clears the word), and
    with the defaults back the next call runs the steps correctly."""
    import ctypes

    monkeypatch.setenv("ADSG_BATCH_ENGINE", "0")
    lib = ads.library()
    b = ads.Batch(SMALL[:3])
    assert b.tuning()["engine"] == "persistent"
    rng = np.random.default_rng(17)
    u0 = [rng.uniform(-1, 1, n) for n in b.sizes]
    for i, u in enumerate(u0):
        b.set_state(i, u)
    assert lib.adsg_batch_test_waits(b._h, 1, 4000) == 0
    code = lib.adsg_batch_steps(b._h, 2)
    if code == 0:
        code = lib.adsg_batch_synchronize(b._h)
    assert code == 1004, code  # ADSG_ERR_DEVICE
    assert b"timed out" in lib.adsg_last_error()
    assert lib.adsg_batch_test_waits(b._h, 0, 1 << 26) == 0
    for i, u in enumerate(u0):
        b.set_state(i, u)
    b.steps(2)
    b.synchronize()
    for i, (nd, p, e, dt) in enumerate(SMALL[:3]):
        pr = oracle.Problem([p] * nd, [e] * nd)
        check(f"after a wait timeout {SMALL[i]} 2 steps", oracle.rel_l2(b.get_state(i), pr.heat_steps(u0[i], dt, 2)),
              2 * STEP, oracle_self(pr, u0[i], dt, 2))
    assert lib.adsg_batch_test_waits(None, 0, 1) == -1
    assert lib.adsg_batch_test_waits(b._h, -1, 1) == -2
    assert lib.adsg_batch_test_waits(b._h, 0, 0) == -3
    del ctypes
