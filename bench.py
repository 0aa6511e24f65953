#!/usr/bin/env python3
"""Benchmark of the IGA-ADS explicit heat step on GB300.

Metric: DOF-updates/s of the explicit step (RHS assembly + ADS mass solve,
FP64).  Workload (default): the 3D heat problem with quadratic B-splines on
128^3 elements (130^3 = 2,197,000 dofs), 3-point Gauss, dt = 1e-6.  A "step"
is one explicit time step of the whole grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload heat3d_p2_128|heat2d_p2_32|heat3d_p4_256|batch64|adjoint_p2_96]

Our arm: inputs resident in HBM, every timed step preceded by an L2 flush
(a 512 MiB memset, outside the step's CUDA-event interval), each step one
adsg_heat_step call (heat_3d::step: the three band passes of the RHS and the
three line solves, 6 kernels, replayed from a cached single-step CUDA graph
where the context's tuner found that faster) on one stream; `e2e` times the
reference-facing host entry point (adsg_heat_steps_host: pinned host tensor
in, one step, host tensor out).  `parity` holds the relative L2 error of the
first step from the bench's initial field against the CPU oracle (whole
field) and against the reference's own run of that step (planes and norms
recorded in tests/golden/, where a record exists for the workload).
The reference arm (--impl reference) times the CPU oracle (a C restatement
of the reference's heat step: Galois-style element loop on all host threads,
single-threaded ADS solve) on the same workload, initial field, step count
and warm-up.
The default run's line also carries `other_configs`: the 2D p=2 34^2 grid,
the 3D p=4 260^3 grid, the batched 64-instance set and the adjoint run, each
measured by this script in a child process on the same GPU right after
(--no-other-configs skips them).
Multi-GPU: replicas only (the single-grid step does not shard); each rank
runs its own copy and value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "iga-ads_gb300"))

WORKLOADS = {
    # name: (ndim, p, elements, dt)
    "heat3d_p2_128": (3, 2, 128, 1e-6),
    "heat2d_p2_32": (2, 2, 32, 1e-5),
    "heat3d_p4_256": (3, 4, 256, 1e-6),
    "batch64": None,  # 32 2D + 32 3D instances, seeded sizes and degrees (ads_gb300.batch_specs)
    "adjoint_p2_96": (3, 2, 96, 1e-6),  # kappa field, 200 steps, sqrt(N) checkpoints
}
METRIC = "DOF-updates/s per explicit step (RHS+ADS solve, FP64, <=1e-12 rel L2)"
DATA = "synthetic: L2 projection of prod sin(pi x_d) + seeded SplitMix64 noise in [-1e-2, 1e-2]"
# The reference's own record of the first and last steps of a workload
# (tests/golden/make_golden.py --runs): planes of the state and its norms.
RUN_RECORDS = {"heat3d_p2_128": "run_3d_p2_e128", "heat3d_p4_256": "run_3d_p4_e256"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heat3d_p2_128", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the summaries of the other configurations in the default workload's line")
    ap.add_argument("--adjoint-steps", type=int, default=200,
                    help="steps of the adjoint workload (its configuration has 200; fewer for a profiling run)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def dist_max(x: float, device=None) -> float:
    """Maximum of x over all ranks (x itself without a process group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, steps: int, seconds_per_rank: float, device=None) -> float:
    """Whole-job throughput of N independent replicas: all units over the
    slowest rank's time (each rank runs the same workload)."""
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    return world * units_per_rank * steps / dist_max(seconds_per_rank, device)


def workload_config(name):
    if name == "batch64":
        import ads_gb300 as ads

        specs = ads.batch_specs(seed=0)
        dofs = sum((e + p) ** nd for nd, p, e, _ in specs)
        return {"workload": "64 independent heat simulations (32 2D with 32-512 elements per side, 32 3D with "
                            "16-96, p in {2,3,4} drawn from seed 0), dt=1e-6, one persistent launch per call",
                "instances": len(specs), "dofs": dofs, "dt": 1e-6,
                "specs": [list(x[:3]) for x in specs]}
    nd, p, E, dt = WORKLOADS[name]
    n = E + p
    return {"workload": f"{nd}D heat, p={p}, {E}^{nd} elements ({n}^{nd} = {n ** nd} dofs), "
                        f"{p + 1}-point Gauss, dt={dt:g}",
            "ndim": nd, "p": p, "elements": E, "dofs": n ** nd, "dt": dt}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle: a C restatement of the reference's step)
# ---------------------------------------------------------------------------
def cpu_baseline(cfg, seconds_budget=20.0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle

    nd, p, E, dt = cfg["ndim"], cfg["p"], cfg["elements"], cfg["dt"]
    threads = os.cpu_count() or 1
    pr = oracle.Problem([p] * nd, [E] * nd)
    rng = np.random.default_rng(0)
    u = rng.uniform(-1, 1, pr.size)
    # one step first to size the sample, then as many whole steps as the budget allows
    t0 = time.perf_counter()
    u = pr.heat_steps(u, dt, 1, nthreads=threads)
    t1 = time.perf_counter()
    steps = 1
    per = t1 - t0
    extra = int(max(0, min(50, (seconds_budget - per) // max(per, 1e-9))))
    if extra:
        t0 = time.perf_counter()
        u = pr.heat_steps(u, dt, extra, nthreads=threads)
        t1 = time.perf_counter()
        steps, per = extra, (t1 - t0) / extra
    return {"value": cfg["dofs"] / per, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full step(s) of the benchmark grid; RHS on {threads} threads (element loop + "
                      f"locked scatter), ADS solve single-threaded", "s_per_step": per}


class _OracleDim:
    """One dimension of an oracle problem in the shape ads_gb300.inputs reads
    (its tables are the oracle's, bit-identical to the reference's)."""

    def __init__(self, pr, d):
        self.p, self.elements = pr.p[d], pr.elements[d]
        self.quad_order = self.p + 1
        self._t = pr.dim(d)

    def dofs(self):
        return self.elements + self.p

    def tables(self):
        return self._t

    def form_band(self, which):
        assert which == 0
        return self._t["mass"].reshape(self.dofs(), 3 * self.p + 1)


def run_reference(args, cfg):
    """The reference arm: the CPU oracle's heat step on all host threads, on
    the same grid, initial field, warm-up and step count as our arm."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from ads_gb300 import inputs  # host-side numpy only (the engine library is not loaded)

    nd, p, E, dt = cfg["ndim"], cfg["p"], cfg["elements"], cfg["dt"]
    threads = os.cpu_count() or 1
    pr = oracle.Problem([p] * nd, [E] * nd)
    u = inputs.initial_field([_OracleDim(pr, d) for d in range(nd)], seed=0)
    t0 = time.perf_counter()
    if args.warmup:
        u = pr.heat_steps(u, dt, args.warmup, nthreads=threads)
    warm = time.perf_counter() - t0
    t0 = time.perf_counter()
    u = pr.heat_steps(u, dt, args.steps, nthreads=threads)
    el = time.perf_counter() - t0
    v = cfg["dofs"] * args.steps / el
    line = {"metric": METRIC, "value": v, "unit": "DOF-updates/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": dict(cfg), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "DOF-updates/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full steps of the benchmark grid after {args.warmup} warm-up "
                                       f"steps ({warm:.1f} s); the CPU oracle restating the reference step, RHS "
                                       f"on {threads} threads, ADS solve single-threaded"},
            "e2e": {"value": v, "unit": "DOF-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def fp64_peak_tflops(torch, dev):
    """cuBLAS DGEMM throughput (best of 5), the FP64 roof used for the roofline."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# DRAM bytes per dof of each step kernel, from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch over the workload's dofs); the captures,
# their commands and the kernels are listed in profiles/traffic_per_dof.md.
# A workload without its own figures takes those of the larger-than-L2
# heat3d_p4_256 workload, where every stage streams whole tensors and the
# traffic grows with the dofs.
NCU_TRAFFIC_PER_DOF = {
    "heat3d_p2_128": {"rhs_outer": 8.1, "rhs_middle": 16.8, "rhs_x": 16.0, "solve_x": 8.0, "solve_y": 8.0,
                      "solve_z": 8.0},
    "heat3d_p4_256": {"rhs_outer": 21.2, "rhs_middle": 29.8, "rhs_x": 22.3, "solve_x": 12.4, "solve_y": 17.2,
                      "solve_z": 17.1},
}


def profiled_traffic(stage, dofs, workload):
    """DRAM bytes of one launch of a stage from the ncu figures above; None
    when the stage has none."""
    per_dof = NCU_TRAFFIC_PER_DOF.get(workload, NCU_TRAFFIC_PER_DOF["heat3d_p4_256"]).get(stage)
    return None if per_dof is None else per_dof * dofs


def step_parity(ctx, u0, cfg, workload, threads):
    """Relative L2 error of one step from u0 (the bench's initial field)
    against the CPU oracle's step (whole field; skipped where one oracle step
    would take minutes) and against the reference's own run of that step
    (planes and norms of its record), scaled by the largest entry."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    nd, p, E, dt = cfg["ndim"], cfg["p"], cfg["elements"], cfg["dt"]
    got = u0.copy()
    ctx.heat_steps_host(got, dt, 1)
    out = {"steps": 1, "tol": 1e-12, "initial_field": "the bench's (seed 0)"}
    if (p + 1) ** (2 * nd) * E ** nd <= 4e9:  # element-loop work of one oracle step
        t0 = time.perf_counter()
        ref = oracle.Problem([p] * nd, [E] * nd).heat_steps(u0, dt, 1, nthreads=threads)
        out["rel_l2_vs_oracle"] = oracle.rel_l2(got, ref)
        out["oracle_s"] = time.perf_counter() - t0
    rec = RUN_RECORDS.get(workload)
    path = os.path.join(ROOT, "tests", "golden", f"{rec}.npz") if rec else None
    if path and os.path.exists(path):
        g = np.load(path)
        n = E + p
        if abs(np.linalg.norm(u0) - float(g["u0_norm"])) <= 1e-14 * float(g["u0_norm"]):
            t = got.reshape(n, n, n)
            out["rel_l2_vs_reference_plane"] = oracle.rel_l2(t[int(g["plane_z_index"])], g["u1_plane_z"])
            out["reference_record"] = f"tests/golden/{rec}.npz (z-plane {int(g['plane_z_index'])})"
            # the same step by the reference's other CPU forms, where recorded
            # (its executor on another thread count, the sequential loop): the
            # bound is twice their largest disagreement where that exceeds the
            # contract, as in the parity tests
            forms = [g] + [np.load(f) for f in (path[:-4] + "_self.npz", path[:-4] + "_oracle_seq.npz")
                           if os.path.exists(f)]
            if len(forms) > 1:
                spread = max(oracle.rel_l2(a["u1_plane_z"], b["u1_plane_z"]) for k, a in enumerate(forms)
                             for b in forms[k + 1:])
                out["cpu_forms_spread"] = spread
                out["tol"] = max(out["tol"], 2 * spread)
                out["tol_note"] = ("twice the largest disagreement among the reference's CPU forms of this step "
                                   "(executor on 8 and 4 threads, sequential loop; z-plane), where above 1e-12")
    return out


def run_ours(args, cfg):
    import numpy as np
    import torch

    import ads_gb300 as ads
    from ads_gb300 import inputs

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nd, p, E, dt = cfg["ndim"], cfg["p"], cfg["elements"], cfg["dt"]

    dims = [ads.Dimension(p, E) for _ in range(nd)]
    ctx = ads.Context(dims)
    u0 = inputs.initial_field(dims, seed=rank)
    A = torch.from_numpy(u0).to(dev)
    B = torch.empty_like(A)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    size = ctx.size
    torch.cuda.synchronize()
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream)  # the flush, the events and our kernels share one stream

    def step(prev, nxt):
        ctx.heat_step(prev, nxt, dt)  # heat_3d::step: compute_rhs, then ads_solve

    # warm-up
    bufs = [A, B]
    for i in range(max(args.warmup, 3)):
        step(bufs[i % 2], bufs[(i + 1) % 2])
    torch.cuda.synchronize()

    peak_fp64 = fp64_peak_tflops(torch, dev)

    def timed_steps(with_stage_timers):
        """K steps, each bracketed by CUDA events on the launching stream with
        an L2 flush before it; returns the summed step time in ms."""
        ctx.stage_times()  # reset
        ctx.enable_stage_timers(with_stage_timers)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for i in range(args.steps):
                flush.zero_()
                starts[i].record(stream)
                step(bufs[i % 2], bufs[(i + 1) % 2])
                ends[i].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ctx.enable_stage_timers(False)
        return sum(s.elapsed_time(e) for s, e in zip(starts, ends))

    sampler = ClockSampler(int(os.environ.get("ADSG_NVSMI_INDEX", local)))
    sampler.start()
    time.sleep(0.3)
    w0 = time.perf_counter()
    # the headline: K plain steps (no events between the step's kernels)
    step_ms = dist_max(timed_steps(False), dev)
    wall = time.perf_counter() - w0
    # the same K steps again with the library's per-kernel timers, for the
    # stage breakdown and the roofline of the dominant kernel
    staged_ms = dist_max(timed_steps(True), dev)
    clocks = sampler.stop()
    stage = ctx.stage_times()
    value = replica_throughput(size, args.steps, step_ms * 1e-3, dev)

    # --- element-wise sum-factorised quadrature (the general RHS path), timed alone ---
    elem = None
    if nd >= 2:
        ctx.enable_stage_timers(True)
        ctx.stage_times()
        for _ in range(3):
            ctx.heat_rhs_elem(bufs[0], bufs[1], dt)
        ctx.stage_times()
        for _ in range(5):
            ctx.heat_rhs_elem(bufs[0], bufs[1], dt)
        t = ctx.stage_times()["rhs_elem"]
        fl = ctx.stage_work()["rhs_elem"][0]
        elem = {"avg_us": 1e3 * t[0] / t[1], "tflops": fl / (t[0] / t[1] * 1e-3) / 1e12,
                "gflop_per_launch": fl / 1e9, "note": "(p+1)^d colour launches per evaluation"}
        # the same with a diffusion field kappa (the adjoint's forward operator)
        kap = torch.from_numpy(inputs.kappa_field(dims, seed=12)).to(dev)
        for _ in range(3):
            ctx.heat_rhs_elem(bufs[0], bufs[1], dt, kappa=kap)
        ctx.stage_times()
        for _ in range(5):
            ctx.heat_rhs_elem(bufs[0], bufs[1], dt, kappa=kap)
        t = ctx.stage_times()["rhs_elem"]
        elem["kappa_avg_us"] = 1e3 * t[0] / t[1]
        if nd == 3:
            # the same field evaluated once at the Gauss points (as a time loop
            # or the adjoint does), then the RHS from those values: same bits
            kq = torch.empty(ctx.kappa_points_count(), dtype=torch.float64, device=dev)
            ctx.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.kappa_points(kap, kq)
            b.record(stream)
            b.synchronize()
            elem["kappa_points_setup_us"] = 1e3 * a.elapsed_time(b)
            for _ in range(3):
                ctx.heat_rhs_elem_points(bufs[0], bufs[1], dt, kq)
            ctx.stage_times()
            for _ in range(5):
                ctx.heat_rhs_elem_points(bufs[0], bufs[1], dt, kq)
            t = ctx.stage_times()["rhs_elem"]
            elem["kappa_points_avg_us"] = 1e3 * t[0] / t[1]
            del kq
        del kap
    ctx.enable_stage_timers(False)

    # --- e2e: the reference-facing host entry point with pinned host buffers ---
    ctx.set_stream(None)
    ke = min(args.steps, 200)
    host = torch.from_numpy(u0.copy()).pin_memory()
    hnp = host.numpy()
    ctx.heat_steps_host(hnp, dt, 1)  # warm the host path
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke):
        ctx.heat_steps_host(hnp, dt, 1)
    e2e_s = dist_max(time.perf_counter() - t0, dev)
    e2e = replica_throughput(size, ke, e2e_s, dev)

    # --- roofline of the dominant kernel ---
    work = ctx.stage_work()
    per_stage = {}
    for name, (ms, n) in stage.items():
        if n:
            fl, by = work[name]
            avg = ms / n
            per_stage[name] = {"launches": n, "avg_us": 1e3 * avg, "share": 0.0,
                               "fp64_slot_gflop_per_launch": fl / 1e9,
                               "fp64_slot_tflops": fl / (avg * 1e-3) / 1e12,
                               "gbs": by / (avg * 1e-3) / 1e9}
    tot = sum(v["avg_us"] * v["launches"] for v in per_stage.values())
    for v in per_stage.values():
        v["share"] = v["avg_us"] * v["launches"] / tot
    dom = max(per_stage, key=lambda k: per_stage[k]["share"])
    d = per_stage[dom]
    peaks = measured_peaks()
    roof = {"bound": "fp64", "kernel": dom, "achieved": d["fp64_slot_tflops"], "peak": peak_fp64, "unit": "TFLOP/s",
            "frac": d["fp64_slot_tflops"] / peak_fp64,
            "achieved_counts": "FP64 issue slots x 2 per second (an FMA, multiply or add each takes one DFMA slot), "
                               "not an IEEE flop count",
            "traffic": profiled_traffic(dom, size, args.workload),
            "peak_source": "cuBLAS DGEMM 4096^3 measured live in bench.py (GB300 FP64 is not in "
                           "MEASURED_PEAKS.json)",
            "flop_convention": "FP64 operations of the implemented algorithm (pair sums on symmetric band rows, "
                               "unit-diagonal two-ended sweeps), 2 flops per FMA, multiply or add: each takes "
                               "one DFMA issue slot, so frac reads as FP64 pipe utilisation against DGEMM",
            "algorithmic_bytes_per_launch": work[dom][1], "hbm_gbs": d["gbs"],
            "hbm_frac_of_measured": d["gbs"] / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None}
    step_flops = sum(work[k][0] * per_stage[k]["launches"] for k in per_stage) / args.steps

    line = {
        "metric": METRIC, "value": value, "unit": "DOF-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": step_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA,
        "config": dict(cfg),
        "timing": {"l2": "flushed before every timed step (512 MiB memset outside the step interval)",
                   "parallelism": f"replicas x{world}"},
        "tuning": {"solve_variants": ctx.solve_variants(), "step_solve_variants": ctx.step_solve_variants(),
                   "launch_pdl": ctx.launch_pdl(), "fused_x": ctx.fused_x(), "step_1block": ctx.step_1block(),
                   "step_cluster": ctx.step_cluster(), "step_graphs": ctx.step_graphs(), "rhs": "factored quadrature (1D Gauss-assembled bands)"},
        "e2e": {"value": e2e, "unit": "DOF-updates/s", "h2d_bytes_per_step": 8 * size, "d2h_bytes_per_step": 8 * size,
                "steps": ke, "entry": "adsg_heat_steps_host"},
        "gpu_launches": sum(v["launches"] for v in per_stage.values()),
        "roofline": roof,
        "stages": per_stage,
        "stage_pass": {"note": "per-kernel CUDA events, a second pass of the same K steps right after the timed one",
                       "ms_per_step": staged_ms / args.steps},
        "element_rhs": elem,
        "step_fp64_slot_tflops": step_flops / (step_ms / args.steps * 1e-3) / 1e12,
        "clocks": clocks,
        "wall_s": wall,
    }
    if rank == 0 and world == 1:
        line["parity"] = step_parity(ctx, u0, cfg, args.workload, os.cpu_count() or 1)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg)
    if rank == 0 and world == 1 and args.workload == "heat3d_p2_128" and not args.no_other_configs:
        ctx.close()
        line["other_configs"] = other_configs(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batch(args, cfg):
    """Batched form: all 64 instances advance `steps` steps through the engine
    the batch chose at creation (one persistent launch, or a graph of
    concurrent per-instance step chains), timed against looping the plain
    per-instance steps one instance after the other over the same states."""
    import numpy as np
    import torch

    import ads_gb300 as ads
    from ads_gb300 import inputs

    torch.cuda.set_device(0)
    specs = ads.batch_specs(seed=0)
    b = ads.Batch(specs)
    for i, (nd, p, e, _) in enumerate(specs):
        dims = [ads.Dimension(p, e) for _ in range(nd)]
        b.set_state(i, inputs.initial_field(dims, seed=1000 + i))
    dofs = sum(b.sizes)
    k = max(1, args.steps)
    b.steps(max(args.warmup, 3))
    b.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the batch runs on its own (blocking) stream, ordered with the default stream's events
    torch.cuda.synchronize()
    e0.record()
    b.steps(k)
    e1.record()
    b.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop()
    kl = max(1, min(k, 20))
    b.steps_looped(1)  # creates the per-instance contexts (autotuned) outside the timing
    b.synchronize()
    torch.cuda.synchronize()
    e0.record()
    b.steps_looped(kl)
    e1.record()
    b.synchronize()
    torch.cuda.synchronize()
    ms_loop = e0.elapsed_time(e1)
    value = dofs * k / (ms * 1e-3)
    loop_value = dofs * kl / (ms_loop * 1e-3)
    # the engine the batch did not choose, timed the same way on its own batch
    chosen = b.tuning()["engine"]
    other = "persistent" if chosen == "concurrent" else "concurrent"
    saved = os.environ.get("ADSG_BATCH_ENGINE")
    os.environ["ADSG_BATCH_ENGINE"] = "0" if other == "persistent" else "1"
    try:
        bo = ads.Batch(specs)
    finally:
        if saved is None:
            os.environ.pop("ADSG_BATCH_ENGINE", None)
        else:
            os.environ["ADSG_BATCH_ENGINE"] = saved
    for i, (nd, p, e, _) in enumerate(specs):
        bo.set_state(i, inputs.initial_field([ads.Dimension(p, e) for _ in range(nd)], seed=1000 + i))
    bo.steps(max(args.warmup, 3))
    bo.synchronize()
    torch.cuda.synchronize()
    e0.record()
    bo.steps(k)
    e1.record()
    bo.synchronize()
    torch.cuda.synchronize()
    ms_other = e0.elapsed_time(e1)
    engines = {chosen: {"value": value, "ms_per_step": ms / k},
               other: {"value": dofs * k / (ms_other * 1e-3), "ms_per_step": ms_other / k,
                       "tuning": bo.tuning()}}
    bo.close()
    line = {"metric": METRIC + " [batched form]", "value": value, "unit": "DOF-updates/s", "n_gpus": 1,
            "steps": k, "warmup": max(args.warmup, 3), "ms_per_step": ms / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: per-instance sin projection + seeded noise",
            "config": {**{kk: v for kk, v in cfg.items() if kk != "specs"}, "tuning": b.tuning(),
                       "l2": "working set larger than L2 (all instances' state and scratch)"},
            "looped_plain_kernels": {"value": loop_value, "ms_per_step": ms_loop / kl, "steps": kl},
            "speedup_vs_loop": value / loop_value,
            "engines": engines,
            "gpu_launches": (k * sum(6 if nd == 3 else 4 for nd, _, _, _ in specs)
                             if b.tuning()["engine"] == "concurrent" else 1),
            "clocks": clocks}
    print(json.dumps(line), flush=True)
    b.close()
    return 0


def run_adjoint(args, cfg):
    """Reverse mode: forward 200 steps (--adjoint-steps) of the kappa-weighted step with sqrt(N)
    checkpoints, mass-norm loss against a second seeded field, gradients with
    respect to u0 and kappa; checked by central differences along 16 seeded
    directions (8 in u0, 8 in kappa) and the dot-product identity."""
    import numpy as np
    import torch

    import ads_gb300 as ads
    from ads_gb300 import inputs

    torch.cuda.set_device(0)
    nd, p, E, dt = cfg["ndim"], cfg["p"], cfg["elements"], cfg["dt"]
    nsteps = max(1, args.adjoint_steps)
    dims = [ads.Dimension(p, E) for _ in range(nd)]
    ctx = ads.Context(dims)
    adj = ads.Adjoint(ctx, nsteps, dt)
    dev = lambda a: torch.from_numpy(a).cuda()
    u0 = dev(inputs.initial_field(dims, seed=11))
    kappa = dev(inputs.kappa_field(dims, seed=12))
    target = dev(inputs.initial_field(dims, seed=13))
    uT, scratch, dL, gu, gk = (torch.empty_like(u0) for _ in range(5))

    def forward(u, k):
        adj.forward(u, k, uT)
        return ads.mass_loss(ctx, uT, target, scratch, dL)

    forward(u0, kappa)  # warm-up (also compiles nothing: all kernels are prebuilt)
    adj.backward(dL, gu, gk)
    ctx.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    torch.cuda.synchronize()
    e[0].record()
    adj.forward(u0, kappa, uT)
    e[1].record()
    torch.cuda.synchronize()
    loss = ads.mass_loss(ctx, uT, target, scratch, dL)
    torch.cuda.synchronize()
    e[2].record()
    adj.backward(dL, gu, gk)
    e[3].record()
    torch.cuda.synchronize()
    t_fwd = e[0].elapsed_time(e[1])
    t_bwd = e[2].elapsed_time(e[3])
    # finite differences along seeded directions (central, exact for the u0 part)
    fd = []
    rng = np.random.default_rng(2024)
    for i in range(16):
        which = "u0" if i < 8 else "kappa"
        d = dev(rng.standard_normal(ctx.size))
        h = 1e-4
        if which == "u0":
            lp, lm = forward(u0 + h * d, kappa), forward(u0 - h * d, kappa)
            an = float(gu @ d)
        else:
            lp, lm = forward(u0, kappa + h * d), forward(u0, kappa - h * d)
            an = float(gk @ d)
        num = (lp - lm) / (2 * h)
        fd.append(abs(num - an) / max(abs(num), abs(an), 1e-300))
    # dot-product identity of the linear map u0 -> u(T)
    x, y = dev(rng.standard_normal(ctx.size)), dev(rng.standard_normal(ctx.size))
    adj.forward(x, kappa, uT)
    lhs = float(uT @ y)
    adj.backward(y, gu, gk)
    ctx.synchronize()
    rhs = float(x @ gu)
    every, count = adj.checkpoints()
    # the same gradient with every state kept (no recomputation): nsteps states
    # of ctx.size doubles, 1.5 GB at 98^3 x 200, against 288 GB of HBM
    adj_all = ads.Adjoint(ctx, nsteps, dt, checkpoint_every=1)
    adj_all.forward(u0, kappa, uT)
    adj_all.backward(dL, gu, gk)
    torch.cuda.synchronize()
    e[0].record()
    adj_all.forward(u0, kappa, uT)
    e[1].record()
    torch.cuda.synchronize()
    ads.mass_loss(ctx, uT, target, scratch, dL)
    torch.cuda.synchronize()
    e[2].record()
    adj_all.backward(dL, gu, gk)
    e[3].record()
    torch.cuda.synchronize()
    t_fwd_all, t_bwd_all = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    adj_all.close()
    dofs = ctx.size
    line = {"metric": METRIC + " [adjoint form]", "value": dofs * nsteps / (t_fwd * 1e-3), "unit": "DOF-updates/s",
            "n_gpus": 1, "steps": nsteps, "warmup": 1, "ms_per_step": t_fwd / nsteps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: sin projection + seeded noise (u0, target), 8-mode seeded Fourier kappa in [0.5, 1.5]",
            "config": {**cfg, "nsteps": nsteps, "checkpoint_every": every, "checkpoints": count,
                       "rhs": "element-wise sum-factorised quadrature with kappa"},
            "forward_ms": t_fwd, "gradient_ms": t_bwd, "gradient_over_forward": t_bwd / t_fwd,
            "all_states_kept": {"checkpoint_every": 1, "state_bytes": 8 * dofs * nsteps, "forward_ms": t_fwd_all,
                                "gradient_ms": t_bwd_all, "gradient_over_forward": t_bwd_all / t_fwd_all},
            "loss": loss, "fd_max_rel_err": max(fd), "fd_rel_errs": fd,
            "dot_product_rel_err": abs(lhs - rhs) / max(abs(lhs), abs(rhs))}
    print(json.dumps(line), flush=True)
    return 0


OTHER_CONFIGS = ("heat2d_p2_32", "heat3d_p4_256", "batch64", "adjoint_p2_96")


def other_configs(args):
    """The other configurations, each measured by this script in a child
    process on the same GPU right after the default workload, summarised
    for the default line: the 2D p=2 34^2 grid, the 3D p=4 260^3 grid, the
    batched 64-instance set and the adjoint run."""
    out = {}
    for w in OTHER_CONFIGS:
        cmd = [sys.executable, os.path.abspath(__file__), "--workload", w, "--steps", str(args.steps), "--warmup",
               str(args.warmup), "--no-cpu-baseline", "--no-other-configs"]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
            d = json.loads(r.stdout.strip().splitlines()[-1])
        except (subprocess.TimeoutExpired, ValueError, IndexError) as e:
            out[w] = {"error": f"{type(e).__name__}: {e}"[:300]}
            continue
        keep = {k: d[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "clocks") if k in d}
        keep["config"] = {k: v for k, v in d.get("config", {}).items() if k != "specs"}
        if "e2e" in d:
            keep["e2e"] = d["e2e"]["value"]
        if "roofline" in d:
            keep["roofline"] = {k: d["roofline"].get(k) for k in ("kernel", "achieved", "peak", "frac", "unit")}
        for k in ("parity", "speedup_vs_loop", "engines", "looped_plain_kernels", "forward_ms", "gradient_ms",
                  "gradient_over_forward", "all_states_kept", "fd_max_rel_err", "dot_product_rel_err",
                  "element_rhs", "tuning", "gpu_launches"):
            if k in d:
                keep[k] = d[k]
        keep["wall_s"] = time.perf_counter() - t0
        out[w] = keep
    return out


def main():
    args = parse()
    cfg = workload_config(args.workload)
    if args.workload == "adjoint_p2_96":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint; its CPU step is "
                              "benchmarked on the single-grid workloads"}))
            return 0
        return run_adjoint(args, cfg)
    if args.workload == "batch64":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched form; its CPU "
                              "step is benchmarked on the single-grid workloads"}))
            return 0
        return run_batch(args, cfg)
    if args.impl == "reference":
        return run_reference(args, cfg)
    return run_ours(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
