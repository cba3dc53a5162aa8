"""Ensembles of source scenarios: the batched solver against one-at-a-time
solves of the same scenarios.

    python cliffs-src_gb300/ensemble.py [--scenarios 256] [--steps 200] [--seed 0]

The ensemble follows the shape of a tsunami source study: scenarios on grids
whose side is drawn from {256, 384, 512, 768, 1024} nodes at 100 m spacing
(the shelf/slope bathymetry of workloads.shelf_2d, one per side), each with
its own seeded source (amplitude 0.5-5 m, half-widths 10-40 % of the domain,
any angle, dipole ratio 0-0.5) applied on the device, 32 gauges per scenario.
Both runs time `steps` steps of every scenario (host clock around the calls,
synchronised) and report
scenarios per second for a 2000-step run (the per-step time times 2000); the
batched run first lets the autotuner pick its plan.  Prints one JSON line.
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


def run(n=256, steps=200, seed=0):
    import torch

    base = bathymetries(seed)
    scs = scenarios(n, seed)
    cells = sum(sc["side"] ** 2 for sc in scs)
    # ---- batched
    grids = [make_grid(base[sc["side"]], sc) for sc in scs]
    b = pkg.Batch(grids)
    tune_ms = b.autotune(4)
    plan = b.plan()
    b.step(2)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.step(steps)
    t_batch = time.perf_counter() - t0
    launches = b.launches()
    maxe = [g.maxwave()[0] for g in grids[:4]]
    b.close()
    for g in grids:
        g.close()
    del grids
    # ---- one at a time: each scenario's own grid, its own launches
    t_seq = 0.0
    for sc in scs:
        g = make_grid(base[sc["side"]], sc)
        g.step(2)
        g.sync()
        t1 = time.perf_counter()
        g.step(steps)
        g.sync()
        t_seq += time.perf_counter() - t1
        g.close()
    ms_b = 1e3 * t_batch / steps
    ms_s = 1e3 * t_seq / steps
    return dict(scenarios=n, steps_timed=steps, cells_total=int(cells), mean_cells=cells / n,
                plan=plan, autotune_ms_per_step=round(tune_ms, 4),
                batched_ms_per_step=round(ms_b, 4), sequential_ms_per_step=round(ms_s, 4),
                batched_scenarios_per_s=round(n / (ms_b * RUN_STEPS / 1e3), 3),
                sequential_scenarios_per_s=round(n / (ms_s * RUN_STEPS / 1e3), 3),
                speedup=round(ms_s / ms_b, 3),
                batched_gcell_per_s=round(cells / (ms_b / 1e3) / 1e9, 2),
                sequential_gcell_per_s=round(cells / (ms_s / 1e3) / 1e9, 2),
                batch_launches=launches, sample_maxe=[float(np.max(m)) for m in maxe])


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
