"""Ensembles of source scenarios: the batched solver against one-at-a-time
solves of the same scenarios.

    python cliffs-src_gb300/ensemble.py [--scenarios 256] [--steps 200] [--seed 0]

The ensemble follows the shape of a tsunami source study: scenarios on grids
whose side is drawn from {256, 384, 512, 768, 1024} nodes at 100 m spacing
(the shelf/slope bathymetry of workloads.shelf_2d, one per side), each with
its own seeded source (amplitude 0.5-5 m, half-widths 10-40 % of the domain,
any angle, dipole ratio 0-0.5) applied on the device, 32 gauges per scenario.
Both runs time `steps` steps of every scenario (host clock around the calls,
synchronised), sampling every scenario's 32 gauges every 10 steps, and
report scenarios per second for a 2000-step run (the per-step time times
2000); the batched run first lets the autotuner pick its plan (schedule and
tile shape).  Prints one JSON line.
"""
import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads

SIDES = (256, 384, 512, 768, 1024)
DX = 100.0
RUN_STEPS = 2000


def scenarios(n, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        side = int(rng.choice(SIDES))
        L = side * DX
        out.append(dict(side=side, x0=rng.uniform(0.2, 0.6) * L, y0=rng.uniform(0.2, 0.8) * L,
                        ax=rng.uniform(0.1, 0.4) * L, ay=rng.uniform(0.1, 0.4) * L,
                        angle=rng.uniform(0, np.pi), amp=rng.uniform(0.5, 5.0),
                        dipole=rng.uniform(0.0, 0.5)))
    return out


def bathymetries(seed=0):
    return {s: W.shelf_2d(seed=seed + s, nx=s, ny=s, dx=DX, steps=0, amp=0.0, ngauges=32) for s in SIDES}


def make_grid(base, sc):
    g = pkg.GpuGrid.from_case(dict(base, H0=base["dep"]))
    g.add_source(base["xcrd"], base["ycrd"], x0=sc["x0"], y0=sc["y0"], ax=sc["ax"], ay=sc["ay"],
                 angle=sc["angle"], amp=sc["amp"], dipole=sc["dipole"])
    return g


def run(n=256, steps=200, seed=0, warmup=2, gout=10, probe_steps=32, sequential=True):
    """Time `steps` steps of every scenario batched (after the autotuner and
    `warmup` steps), and one at a time; the 32 gauges of every scenario are
    sampled every `gout` steps in both runs (cliffs_batch_get_gauges, one
    launch for all scenarios; asynchronous gauge records per grid,
    cliffs_gpu_get_gauges_async).  Host clock around calls that
    synchronise."""
    import torch

    base = bathymetries(seed)
    scs = scenarios(n, seed)
    cells = sum(sc["side"] ** 2 for sc in scs)
    gauges = [base[sc["side"]]["gauges"] for sc in scs]
    m = sum(len(I) for I, _ in gauges)
    rec = [pkg.cliffs_gpu.pinned((m,)) for _ in range(3)]
    # ---- batched
    grids = [make_grid(base[sc["side"]], sc) for sc in scs]
    b = pkg.Batch(grids)
    b.set_gauges(gauges)
    tune_ms = b.autotune(probe_steps)
    plan = b.plan()
    b.step(warmup)
    torch.cuda.synchronize()
    l0 = b.launches()
    t0 = time.perf_counter()
    for s0 in range(0, steps, gout):
        b.step(min(gout, steps - s0))
        b.gauges(out=rec)
    t_batch = time.perf_counter() - t0
    launches = b.launches() - l0
    maxe = [g.maxwave()[0] for g in grids[:4]]
    status = [g.status()[0] for g in grids]
    b.close()
    for g in grids:
        g.close()
    del grids
    out = dict(scenarios=n, steps_timed=steps, gauges_every=gout, gauges_total=m, cells_total=int(cells),
               mean_cells=cells / n, plan=plan, autotune_ms_per_step=round(tune_ms, 4),
               batched_ms_per_step=round(1e3 * t_batch / steps, 4),
               batched_scenarios_per_s=round(n / (t_batch / steps * RUN_STEPS), 3),
               batched_gcell_per_s=round(cells * steps / t_batch / 1e9, 2),
               batch_launches=launches, sample_maxe=[float(np.max(x)) for x in maxe],
               status_ok=all(r == 0 for r in status))
    if not sequential:
        return out
    # ---- one at a time: each scenario's own grid, its own step graphs
    t_seq = 0.0
    for sc in scs:
        g = make_grid(base[sc["side"]], sc)
        I, J = base[sc["side"]]["gauges"]
        g.set_graph_steps(gout)
        g.step(warmup)
        g.prepare_steps(gout)
        g.sync()
        grec = pkg.cliffs_gpu.pinned((3, len(I)))
        t1 = time.perf_counter()
        last = -1
        for s0 in range(0, steps, gout):
            g.step(min(gout, steps - s0))
            last = g.gauges_async(I, J, (grec[0], grec[1], grec[2]))
        g.wait(last)
        g.sync()
        t_seq += time.perf_counter() - t1
        g.close()
    out.update(sequential_ms_per_step=round(1e3 * t_seq / steps, 4),
               sequential_scenarios_per_s=round(n / (t_seq / steps * RUN_STEPS), 3),
               sequential_gcell_per_s=round(cells * steps / t_seq / 1e9, 2),
               speedup=round(t_seq / t_batch, 3))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenarios", type=int, default=256)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    pkg.build.build()
    print(json.dumps(run(a.scenarios, a.steps, a.seed)), flush=True)


if __name__ == "__main__":
    main()
