"""The multi-GPU path of bench.py is replicas only: each rank runs its own
copy of the step and the job's throughput is all ranks' units over the
slowest rank's time.  Checked with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    seconds = [2.0, 3.0][rank]
    out[rank] = (bench.dist_max(seconds), bench.replica_throughput(1000.0, 10, seconds))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_sum_over_slowest():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        mx, thr = out[r]
        assert mx == 3.0
        assert thr == pytest.approx(2 * 1000.0 * 10 / 3.0)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_max(1.5) == 1.5
    assert bench.replica_throughput(10.0, 3, 2.0) == 15.0
