"""A second CPU form of a full-size 3D run: the oracle's executor (all host
threads) over the same steps, from the same initial field, as the
reference's own run recorded by make_golden.py --runs, with the same
snapshot (planes after the first and the last step, the L2 and mass norms).
How far the two CPU forms of the reference's algorithm drift apart over the
run bounds the GPU's drift from the reference (tests/test_gpu_fullsize.py).

    python tests/golden/oracle_run.py run_3d_p4_e256 [--threads N]
    python tests/golden/oracle_run.py run_3d_p4_e256 --sequential-first-step

writes tests/golden/<name>_oracle.npz (the whole run on the executor), or
<name>_oracle_seq.npz (the first step by the sequential element loop, the
order a reference build without Galois runs).  Needs the oracle (make -C
oracle) and the engine's Python package (for the seeded initial field); not
the reference sources."""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "iga-ads_gb300"))

from make_golden import RUNS, snapshot  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("name", choices=[r[0] for r in RUNS])
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--sequential-first-step", action="store_true",
                    help="only the first step, by the sequential element loop (<name>_oracle_seq.npz)")
    a = ap.parse_args()
    import oracle

    import ads_gb300 as ads
    from ads_gb300 import inputs

    name, p, E, dt, nsteps, seed = next(r for r in RUNS if r[0] == a.name)
    n = E + p
    u = inputs.initial_field([ads.Dimension(p, E) for _ in range(3)], seed=seed)
    pr = oracle.Problem([p] * 3, [E] * 3)
    mass = pr.dim(0)["mass"]
    out = dict(p=np.int32(p), elements=np.int32(E), dt=np.float64(dt), nsteps=np.int32(nsteps), seed=np.int64(seed),
               threads=np.int32(a.threads), u0_norm=np.float64(np.linalg.norm(u)))
    t0 = time.time()
    if a.sequential_first_step:
        u = pr.heat_steps(u, dt, 1)
        out.update(snapshot(u, n, mass, p, "u1_", "z"))
        out["threads"] = np.int32(1)
        path = os.path.join(a.out, name + "_oracle_seq.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} after {time.time() - t0:.0f} s", flush=True)
        return
    u = pr.heat_steps(u, dt, 1, nthreads=a.threads)
    out.update(snapshot(u, n, mass, p, "u1_", "z"))
    print(f"{name} (oracle): step 1 done in {time.time() - t0:.0f} s", flush=True)
    u = pr.heat_steps(u, dt, nsteps - 1, nthreads=a.threads)
    out.update(snapshot(u, n, mass, p, "uN_", "zy"))
    out["seconds"] = np.float64(time.time() - t0)
    path = os.path.join(a.out, name + "_oracle.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} after {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main()
