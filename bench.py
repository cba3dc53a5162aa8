"""Benchmark: Cliffs time stepping on the 2048x2048 Cartesian shelf basin.

One step = one time step of the whole grid (x-sweep over all rows, which
also folds the previous step's end state into the max-wave fields, and
y-sweep over all columns), i.e. one pass of the hot path of
cliffs_main.f:303-355.  Metric: Mcell-updates/s = nx*ny*steps/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--kernels-only] [--workload shelf2048|sphere4320] [--sweep tiled|direct|staged]

--kernels-only runs the device-resident passes alone (no end-to-end pass, no
CPU sample): the command the ncu summaries under profiles/ capture.

--workload sphere4320 runs a 4320 x 2160 spherical grid (1/12 degree in
longitude, 80S-80N) instead of the 2048^2 Cartesian shelf, the default and
the benchmark line.

--workload ensemble256 runs the batched ensemble: 256 source scenarios on
grids of 256^2 to 1024^2 cells stepped together (cliffs_batch_*, plan from
the autotuner), 32 gauges per scenario sampled every 10 steps; the metric is
scenarios/s for 2000-step scenarios, beside the same scenarios solved one at
a time (each grid's own step graphs).

--workload surrogate runs the learned-surrogate study: 4096 training runs of
2000 steps on a 512^2 grid from the batched solver, 4 gauge networks (MLP,
3000 epochs) and a map network (MLP and conv decoder, 600 epochs) trained by
the library's kernels, then --steps gated passes over 256 held-out
scenarios against one-at-a-time solves; the metric is scenarios/s of the
gated path (surrogate plus solver fallbacks).

The default line (the shelf, one GPU) also carries "workloads": the other
configurations of the benchmark set, each run whole in its own process after
the shelf's measurements (the batched ensemble of 256 scenarios, the learned
surrogate, the nested spherical chain over 6 model hours), with their own
metrics and baselines; --kernels-only leaves them out.

--impl reference times the CPU restatement of the reference solver (the
Fortran reference cannot be compiled on these hosts) with all host threads on
the same workload.  With N > 1 (torchrun) every rank runs an independent
replica on its own GPU: the plain solver does not shard (replicas only).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = 2048
DX = 100.0
SEED = 0
# algorithmic bytes per cell (FP32) of a two-dimensional step's sweeps
B_X = 44   # x-sweep: read dep,eta,u,v; write eta,u,v; read/write hmax,velmax (the previous step's end state)
B_Y = 28   # y-sweep: read dep,eta,u,v; write eta,u,v
B_STEP = B_X + B_Y
# Steps one run of the workload may take.  In the reference scheme (and the
# FP64 oracle alike) an edge wave running along the east coast reaches the
# corner with the open south boundary and the run goes unstable after ~3900
# steps; every pass here starts from the initial state and stays below that.
HORIZON = 3500


def _env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x, dist):
    """The largest of every rank's x (seconds): the job's time is its slowest
    replica's.  dist is torch.distributed with a process group, or None."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, cells, steps, seconds):
    """Whole-job Mcell-updates/s: every replica's cells and steps over the
    slowest replica's time."""
    return world * cells * steps / seconds / 1e6


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def workload(name="shelf2048"):
    """shelf2048: the benchmark (2048^2 Cartesian shelf basin at 100 m).
    sphere4320: a 4320 x 2160 spherical grid (1/12 degree in longitude,
    80 S to 80 N) on the same bathymetry generator, 37 MB per field."""
    import importlib

    import numpy as np
    W = importlib.import_module("cliffs-src_gb300.workloads")
    if name == "shelf2048":
        case = W.shelf_2d(seed=SEED, nx=NX, ny=NY, dx=DX, steps=3000, ngauges=64)
        case["crough"] = 0.000625  # Manning n = 0.025, as in the reference's Okushiri example
        case["label"] = (f"shelf_2d {NX}x{NY} dx={DX:g} m, FP32 state, runs of at most {HORIZON} steps from the "
                         f"initial state, 64 gauges every 10 steps (end-to-end pass)")
        case["source_label"] = "elliptical Gaussian uplift 100x50 km, 2 m"
        return case
    if name == "sphere4320":
        nx, ny = 4320, 2160
        case = W.sphere_2d(seed=SEED + 3, nx=nx, ny=ny, steps=3000, ngauges=64)
        case["crough"] = 0.000625
        case["label"] = (f"spherical {nx}x{ny}, 1/12 deg in longitude, 80S-80N, FP32 state, runs of at most "
                         f"{HORIZON} steps, 64 gauges every 10 steps (end-to-end pass)")
        case["source_label"] = "elliptical Gaussian uplift, half-axes 30x15 nodes, 2 m"
        return case
    raise ValueError(f"unknown workload {name}")


def config_dict(case):
    """The workload; the same for both arms (the implementation is named
    outside it, under "implementation")."""
    ny, nx = case["dep"].shape
    return {"workload": case["label"], "grid": [nx, ny], "dt_s": round(case["dt"], 6), "ground_m": case["ground"],
            "crough": case["crough"], "source": case["source_label"],
            "l2": f"working set ~{9 * nx * ny * 4 / 1e6:.0f} MB per step > 129 MB L2; no flush",
            "parallelism": "replicas only (one independent grid per GPU)"}


def cpu_baseline(case, steps, threads, f32=True, warmup=1):
    """The CPU restatement (oracle) timed on a bounded sample of the workload;
    with f32, also the same source built in FP32 (like for like with the FP32
    GPU path), reported under "f32"."""
    import oracle  # noqa: F401
    from tests.runners import oracle_model, oracle_model32
    os.environ["OMP_NUM_THREADS"] = str(threads)
    cells = case["dep"].size

    def timed(m):
        m.step(warmup)
        t0 = time.perf_counter()
        m.step(steps)
        return cells * steps / (time.perf_counter() - t0) / 1e6

    val = timed(oracle_model(case))
    line = {"value": round(val, 3), "unit": "Mcell-updates/s", "cores": threads, "kind": "port",
            "sample": f"{case['dep'].shape[1]}x{case['dep'].shape[0]} grid, {steps} time steps after {warmup} "
                      f"warm-up step{'s' if warmup != 1 else ''}, OpenMP over lines ({threads} threads), FP64"}
    if f32:
        line["f32"] = {"value": round(timed(oracle_model32(case)), 3), "unit": "Mcell-updates/s",
                       "sample": "the same steps with the same source built in FP32 (orc_real = float)"}
    return line


def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    # The oracle library reads OMP_NUM_THREADS when it first starts OpenMP.
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle  # noqa: F401  (builds/loads the CPU restatement)
    case = workload(args.workload)
    # a bounded sample: at most 300 timed steps after at most 50 warm-up steps
    # (~28 ms per step on 16 cores)
    steps = max(1, min(args.steps, 300))
    warm = max(1, min(args.warmup, 50))
    cb = cpu_baseline(case, steps, threads, f32=False, warmup=warm)
    line = {"metric": "Mcell-updates/s", "value": cb["value"], "unit": "Mcell-updates/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": round(1e3 * case["dep"].size / (cb["value"] * 1e6), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(case),
            "implementation": "CPU restatement of cliffs.f + cliffs_main.f time loop (oracle, OpenMP)",
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_e2e(pkg, case, args, barrier, dist, world):
    """Steps through the public API from host buffers: create the grid from
    the FP64 bathymetry and metrics, upload the initial state, step, gauge
    records every 10 steps (asynchronous outputs, cliffs_gpu_get_gauges_async),
    final state and max-wave fields back to the host.  The driver's arrays
    (inputs read from its files, outputs it writes) are pinned host memory
    (cliffs_gpu_host_alloc), allocated and filled before the clock starts, as
    a driver that keeps its module arrays there does.  The pass runs twice
    and the second is timed: a process's first call of each kernel loads it
    (CUDA's lazy module loading), which the device-resident passes leave to
    their warm-up steps too."""
    import numpy as np

    cells = case["dep"].size
    ny, nx = case["dep"].shape
    I, J = case["gauges"]
    nrec = (args.steps + 9) // 10
    pin = pkg.cliffs_gpu.pinned
    rec = pin((nrec, 3, len(I)))
    state = [pin((ny, nx)) for _ in range(3)]
    maxes = [pin((ny, nx), np.float32) for _ in range(2)]
    inputs = {}
    for k in ("dep", "H0", "u0", "v0"):
        inputs[k] = pin((ny, nx))
        inputs[k][...] = case[k]

    def one_pass():
        t0 = time.perf_counter()
        dx, rs, dy, zeta = pkg.cliffs_gpu.metrics(case["xcrd"], case["ycrd"], case["cartesian"])
        g2 = pkg.GpuGrid(inputs["dep"], dx=dx, row_scale=rs, dy=dy, zeta=zeta, ground=case["ground"],
                         crough=case["crough"], dt=case["dt"])  # create: bathymetry H2D
        g2.set_initial(inputs["H0"], inputs["u0"], inputs["v0"])  # initial state H2D
        g2.set_graph_steps(10)  # one graph per gauge interval
        last = -1
        for k, s0 in enumerate(range(0, args.steps, 10)):
            g2.step(min(10, args.steps - s0))
            last = g2.gauges_async(I, J, (rec[k, 0], rec[k, 1], rec[k, 2]))
        g2.download_state(out=state)
        g2.maxwave(out=maxes)
        g2.wait(last)
        t = time.perf_counter() - t0
        r, flags = g2.status()
        g2.close()
        if r != 0:
            raise RuntimeError(f"solver status {r} flags {flags} (end-to-end pass)")
        return t

    # one untimed pass first, as the device-resident passes have their
    # warm-up: the first call of each output kernel in a process loads it
    one_pass()
    barrier()
    t_e2e = one_pass()
    t_e2e = max_over_ranks(t_e2e, dist)
    h2d = cells * 8 * 4 + (nx + ny) * 8 * 3 + 64 * 8 * nrec  # dep, H0, u0, v0 (FP64), metrics, gauge indices
    d2h = cells * 8 * 3 + cells * 4 * 2 + nrec * 64 * 3 * 8
    return {"value": round(job_value(world, cells, args.steps, t_e2e), 3), "unit": "Mcell-updates/s",
            "h2d_bytes_per_step": int(h2d // args.steps), "d2h_bytes_per_step": int(d2h // args.steps),
            "ms": round(t_e2e * 1e3, 3), "host_buffers": "pinned (cliffs_gpu_host_alloc)"}


def run_ours(args):
    import importlib

    import numpy as np
    import torch

    rank, world, local = _env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    pkg = importlib.import_module("cliffs-src_gb300")
    pkg.build.build()
    case = workload(args.workload)
    cells = case["dep"].size

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- device-resident throughput (value) ----------------------------------
    stream = torch.cuda.Stream()
    kind = {"tiled": pkg.cliffs_gpu.TILED, "direct": pkg.cliffs_gpu.DIRECT, "staged": pkg.cliffs_gpu.STAGED}[args.sweep]
    g = pkg.GpuGrid.from_case(case)
    g.set_stream(stream.cuda_stream)
    g.set_sweep_kernel(kind)
    g.step(args.warmup)
    # the CUDA graphs the timed call replays are instantiated here, so the
    # timed region launches them only
    g.prepare_steps(args.steps)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        n0 = g.launches()
        e0.record(stream)
        done, _ = g.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        launches = g.launches() - n0
    barrier()
    ms = e0.elapsed_time(e1)
    r, flags = g.status()
    if r != 0:
        raise RuntimeError(f"solver status {r} flags {flags}")
    g.close()
    # ---- per-kernel durations: the same steps again from the initial state,
    # with CUDA events around every sweep on the solver's stream ---------------
    g = pkg.GpuGrid.from_case(case)
    g.set_stream(stream.cuda_stream)
    g.set_sweep_kernel(kind)
    g.step(args.warmup)
    g.profile(True)
    g.step(args.steps)
    prof = g.profile_read()
    g.profile(False)
    r, flags = g.status()
    if r != 0:
        raise RuntimeError(f"solver status {r} flags {flags}")
    g.close()
    t_local = ms / 1e3
    t_max = max_over_ranks(t_local, dist)
    value = job_value(world, cells, args.steps, t_max)

    # ---- end to end through the C ABI with host buffers (e2e) -----------------
    e2e = None
    if not args.kernels_only:
        e2e = run_e2e(pkg, case, args, barrier, dist, world)

    # ---- roofline of the dominant kernel ---------------------------------------
    peak, peak_kind = _peaks()
    kx, ky = prof["x_ms"], prof["y_ms"]
    if args.sweep == "staged":  # the max-wave update stays in the y-sweep
        names = ("x-sweep: staged_x", "y-sweep + max-wave: staged_y")
        bx, by = B_Y, B_X
    else:
        names = ("x-sweep + max-wave of the previous step's end state: fast_kernel<0, true, false>",
                 "y-sweep: tile_y_kernel (tiles in and out by tensor-map copies)" if args.sweep == "tiled"
                 else "y-sweep: fast_kernel<1, true, false>")
        bx, by = B_X, B_Y
    if ky >= kx:
        kname, kms, bpc = names[1], ky, by
    else:
        kname, kms, bpc = names[0], kx, bx
    achieved = bpc * cells / (kms / 1e3) / 1e9 if kms > 0 else 0.0
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tp) and args.sweep == "tiled":
        with open(tp) as f:
            tr = json.load(f)
        key = "y" if ky >= kx else "x"
        tr = tr.get(args.workload, {})
        if key in tr:
            traffic = int(tr[key]["bytes_per_cell"] * cells)
    roof = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
            "bytes_per_cell": bpc, "launch_ms": round(kms, 5), "peak_source": peak_kind,
            "x_ms": round(kx, 5), "y_ms": round(ky, 5)}

    if rank == 0:
        threads = os.cpu_count() or 1
        cb = None if args.kernels_only else cpu_baseline(case, 300, threads)
        clocks = clk.summary()
        line = {"metric": "Mcell-updates/s", "value": round(value, 3), "unit": "Mcell-updates/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(ms / args.steps, 5), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config_dict(case), "implementation": "CUDA sm_103a, include/cliffs_gpu.h",
                "e2e": e2e, "roofline": roof, "cpu_baseline": cb, "clocks": clocks,
                "gpu_launches": int(launches),
                "hbm_frac_step": round(B_STEP * cells * args.steps / (ms / 1e3) / 1e9 / peak, 4)}
        if world == 1 and args.workload == "shelf2048" and not args.kernels_only:
            # this process's cached device memory goes back before the children run
            torch.cuda.empty_cache()
            line["workloads"] = side_workloads()
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_ensemble(args):
    """The batched ensemble line (one GPU; replicas only across GPUs)."""
    import importlib

    import torch

    rank, world, local = _env_rank()
    E = importlib.import_module("cliffs-src_gb300.ensemble")
    n, steps = 256, max(10, args.steps)
    scs = E.scenarios(n, 0)
    cells = sum(sc["side"] ** 2 for sc in scs)
    config = {"workload": f"ensemble of {n} source scenarios, sides drawn from {list(E.SIDES)} at {E.DX:g} m "
                          f"(shelf/slope bathymetry), seeded Gaussian uplifts 0.5-5 m, FP32 state, "
                          f"32 gauges per scenario every 10 steps",
              "scenarios": n, "cells_total": int(cells), "run_steps_per_scenario": E.RUN_STEPS,
              "l2": f"working set ~{9 * cells * 4 / 1e6:.0f} MB per step > 129 MB L2; no flush",
              "parallelism": "replicas only (one independent ensemble per GPU)"}
    if args.impl == "reference":
        if rank != 0:
            return 0
        threads = os.cpu_count() or 1
        cb = ensemble_cpu_baseline(E, scs, threads)
        line = {"metric": "scenarios/s", "value": cb["value"], "unit": cb["unit"], "n_gpus": args.gpus,
                "steps": cb["steps"], "warmup": 1, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "implementation": "CPU restatement of cliffs.f + cliffs_main.f time loop (oracle, OpenMP), "
                                  "one scenario after another",
                "impl": "reference", "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    torch.cuda.set_device(local)
    pkg = importlib.import_module("cliffs-src_gb300")
    pkg.build.build()
    with ClockSampler(local) as clk:
        r = E.run(n, steps, seed=0, warmup=max(3, args.warmup))
    if not r["status_ok"]:
        raise RuntimeError("a scenario reported a non-zero status")
    e2e = ensemble_e2e(pkg, E, n, steps, r["plan"])
    peak, peak_kind = _peaks()
    ms = r["batched_ms_per_step"]
    achieved = B_STEP * cells / (ms / 1e3) / 1e9
    cb = ensemble_cpu_baseline(E, scs, os.cpu_count() or 1) if rank == 0 else None
    line = {"metric": "scenarios/s", "value": r["batched_scenarios_per_s"],
            "unit": f"scenarios/s ({E.RUN_STEPS}-step scenarios)", "n_gpus": world, "steps": steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": dict(config, plan=r["plan"]),
            "implementation": "CUDA sm_103a, include/cliffs_gpu.h cliffs_batch_* (graph or persistent plan)",
            "timing": "host clock around synchronised batch calls (each call ends with a stream synchronise)",
            "sequential": {"ms_per_step": r["sequential_ms_per_step"],
                           "scenarios_per_s": r["sequential_scenarios_per_s"],
                           "what": "the same scenarios one at a time, each grid's steps from its own CUDA "
                                   "graphs, asynchronous gauge records"},
            "speedup_vs_sequential": r["speedup"], "autotune_ms_per_step": r["autotune_ms_per_step"],
            "e2e": e2e,
            "roofline": {"bound": "hbm", "kernel": "batched x- and y-sweep phases and gauges, per step",
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "bytes_per_cell": B_STEP,
                         "peak_source": peak_kind},
            "cpu_baseline": cb, "clocks": clk.summary(), "gpu_launches": int(r["batch_launches"])}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def ensemble_cpu_baseline(E, scs, threads, steps=10):
    """The oracle's time loop on one grid of each side (the ensemble's
    bathymetry and a source of the ensemble), `steps` steps each after one
    warm-up step; the ensemble's time per step is the sum over its
    scenarios of cells / measured rate of that side."""
    import oracle  # noqa: F401
    from tests.runners import oracle_model
    os.environ["OMP_NUM_THREADS"] = str(threads)
    base = E.bathymetries(0)
    rate = {}
    for side in E.SIDES:
        sc = next(s for s in scs if s["side"] == side)
        c = dict(base[side])
        # the source as the GPU applies it (bottom fixed, surface raised)
        c["H0"] = base[side]["dep"] + E.pkg.cliffs_gpu.source_field(
            c["xcrd"], c["ycrd"], x0=sc["x0"], y0=sc["y0"], ax=sc["ax"], ay=sc["ay"], angle=sc["angle"],
            amp=sc["amp"], dipole=sc["dipole"])
        m = oracle_model(c)
        m.step(1)
        t0 = time.perf_counter()
        m.step(steps)
        rate[side] = side * side * steps / (time.perf_counter() - t0)
    t_step = sum(s["side"] ** 2 / rate[s["side"]] for s in scs)
    return {"value": round(len(scs) / (t_step * E.RUN_STEPS), 4),
            "unit": f"scenarios/s ({E.RUN_STEPS}-step scenarios)",
            "cores": threads, "kind": "port", "steps": steps, "ms_per_step": round(1e3 * t_step, 3),
            "sample": f"one grid per side {list(E.SIDES)}, {steps} time steps after 1 warm-up step, OpenMP over "
                      f"lines ({threads} threads), FP64; the ensemble's step time is the sum over its "
                      f"{len(scs)} scenarios of cells / the measured rate of their side",
            "rates_mcell_per_s": {str(k): round(v / 1e6, 1) for k, v in rate.items()}}


def ensemble_e2e(pkg, E, n, steps, plan):
    """The ensemble end to end through the public API: grids created from the
    host's FP64 bathymetry and initial state (pinned arrays), sources applied
    on the device, the batch and its gauges set up, `steps` steps with the
    gauge records every 10 steps, and every scenario's max-wave fields back
    to pinned host arrays.  plan: the device-resident run's plan (the tile
    shape the autotuner chose there, graphs of 10 steps; no autotuning inside
    the timed region).  Unit: 2000-step scenarios per second, with the set-up
    counted once per `steps` steps."""
    import numpy as np

    base = E.bathymetries(0)
    scs = E.scenarios(n, 0)
    pin = pkg.cliffs_gpu.pinned
    host = {}
    for side, c in base.items():
        host[side] = {k: pin(c["dep"].shape) for k in ("dep", "H0")}
        host[side]["dep"][...] = c["dep"]
        host[side]["H0"][...] = c["dep"]
    maxes = [(pin((sc["side"],) * 2, np.float32), pin((sc["side"],) * 2, np.float32)) for sc in scs]
    gauges = [base[sc["side"]]["gauges"] for sc in scs]
    m = sum(len(I) for I, _ in gauges)
    rec = [pin((m,)) for _ in range(3)]
    cells = sum(sc["side"] ** 2 for sc in scs)
    t0 = time.perf_counter()
    grids = []
    for sc in scs:
        c = base[sc["side"]]
        dx, rs, dy, zeta = pkg.cliffs_gpu.metrics(c["xcrd"], c["ycrd"], True)
        g = pkg.GpuGrid(host[sc["side"]]["dep"], dx=dx, row_scale=rs, dy=dy, zeta=zeta, ground=c["ground"],
                        crough=c["crough"], dt=c["dt"])
        g.set_initial(host[sc["side"]]["H0"])
        g.add_source(c["xcrd"], c["ycrd"], x0=sc["x0"], y0=sc["y0"], ax=sc["ax"], ay=sc["ay"],
                     angle=sc["angle"], amp=sc["amp"], dipole=sc["dipole"])
        grids.append(g)
    b = pkg.Batch(grids)
    b.set_gauges(gauges)
    xr, yg = plan.get("x_rows", 1), plan.get("y_groups", 1)
    b.set_plan(pkg.cliffs_gpu.GRAPH, graph_steps=10, x_rows=xr, y_groups=yg)
    for s0 in range(0, steps, 10):
        b.step(min(10, steps - s0))
        b.gauges(out=rec)
    for g, out in zip(grids, maxes):
        g.maxwave(out=out)
    t = time.perf_counter() - t0
    b.close()
    for g in grids:
        g.close()
    h2d = sum(sc["side"] ** 2 * 8 * 2 for sc in scs)
    d2h = sum(sc["side"] ** 2 * 4 * 2 for sc in scs) + (steps // 10) * m * 24
    return {"value": round(n * steps / (E.RUN_STEPS * t), 3), "unit": f"scenarios/s ({E.RUN_STEPS}-step scenarios)",
            "h2d_bytes_per_step": int(h2d // steps), "d2h_bytes_per_step": int(d2h // steps),
            "ms": round(1e3 * t, 1), "gcell_per_s": round(cells * steps / t / 1e9, 2),
            "plan": f"graph of 10 steps, tile shape {xr} x {yg} (no autotuning inside the timed region)"}


def run_surrogate(args):
    """The learned-surrogate line: gated scenarios/s against one-at-a-time
    solves, with the surrogate's errors against the solver."""
    import importlib

    rank, world, local = _env_rank()
    S = importlib.import_module("cliffs-src_gb300.surrogate")
    epochs, map_epochs = 3000, 600
    config = {"workload": f"learned surrogate of {S.SIDE}x{S.SIDE} shelf runs at {S.DX:g} m, 2000 steps each: 8 "
                          f"source parameters -> {S.NGAUGES} gauge maxima and a {S.MAP}x{S.MAP} max-inundation "
                          f"map; 4096 training runs from the batched solver, 256 held-out scenarios; 4 gauge "
                          f"networks (MLP 9 -> 512 x 3 -> 64, {epochs} epochs) and a map network (the same MLP "
                          f"and a conv decoder {list(S.MAP_CH)}, {map_epochs} epochs); a step is one gated pass "
                          f"over the 256 held-out scenarios",
              "parallelism": "replicas only"}
    if args.impl == "reference":
        if rank != 0:
            return 0
        threads = os.cpu_count() or 1
        cb = surrogate_cpu_baseline(S, threads)
        line = {"metric": "scenarios/s", "value": cb["value"], "unit": "scenarios/s", "n_gpus": args.gpus,
                "steps": cb["steps"], "warmup": 1, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "implementation": "CPU restatement of the solver (oracle, OpenMP), one scenario after another",
                "impl": "reference", "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "scenarios/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    import torch
    torch.cuda.set_device(local)
    S.pkg.build.build()
    with ClockSampler(local) as clk:
        D = S.make_data(4096, 256, 2000, 0)
        r = S.fit_and_judge(D, epochs=epochs, map_epochs=map_epochs, target=0.045, members=4, map_members=1,
                            repeats=max(1, args.steps))
    peak = None
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            peak = float(json.load(f)["bf16_tflops"])
    achieved = r["predict_flop"] / (r["predict_ms"] / 1e3) / 1e12  # the gated path's forward products
    cb = surrogate_cpu_baseline(S, os.cpu_count() or 1) if rank == 0 else None
    n_y = S.NGAUGES + S.MAP * S.MAP
    line = {"metric": "scenarios/s", "value": r["gated_scenarios_per_s"], "unit": "scenarios/s", "n_gpus": world,
            "steps": r["repeats"], "warmup": 1, "ms_per_step": round(r["predict_ms"] + r["fallback_solve_ms"], 3),
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 products, fp32 accumulation", "data": "synthetic", "config": config,
            "implementation": "CUDA sm_103a: cliffs_batch_* (data), cliffs_mlp_* (training, inference)",
            "timing": "host clock, medians over the steps; the gated path is the networks' predictions (gauges and "
                      "maps, host arrays in and out) plus one batched solve of the rejected scenarios (grid set-up, "
                      "sources, steps, max-wave download); the warm-up is the gate's calibration pass",
            "infer_scenarios_per_s": r["infer_scenarios_per_s"], "infer_batch": r["infer_batch"],
            "one_at_a_time_scenarios_per_s": r["one_at_a_time_scenarios_per_s"],
            "speedup_vs_one_at_a_time": r["gated_speedup_vs_one_at_a_time"],
            "gauge_rel_err_gated_mean": r["gated_rel_err_mean"],
            "gauge_rel_err_accepted_mean": r["gauge_rel_err_accepted_mean"],
            "map_abs_err_mean_m": r["map_abs_err_mean_m"], "map_iou_mean": r["map_iou_mean"],
            "map_max_depth_rel_err_mean": r["map_max_depth_rel_err_mean"],
            "fallback": r["fallback"], "data_seconds": r["data_seconds"], "train_seconds": r["train_seconds"],
            "e2e": {"value": r["gated_scenarios_per_s"], "unit": "scenarios/s",
                    "h2d_bytes_per_step": 256 * S.N_FEATURES * 4, "d2h_bytes_per_step": 4 * 256 * n_y * 4,
                    "what": "host parameters in, host gauge maxima and maps out (the predictions copy both ways)"},
            "roofline": {"bound": "tensor",
                         "kernel": "the networks' forward passes over the held-out scenarios (tcgen05 products "
                                   "gemm_tc, direct decoder convolutions), host copies included",
                         "achieved": round(achieved, 3), "peak": peak, "unit": "TFLOP/s",
                         "frac": round(achieved / peak, 5) if peak else None, "traffic": None},
            "cpu_baseline": cb, "clocks": clk.summary(), "result": r}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def surrogate_cpu_baseline(S, threads, steps=100):
    """The oracle's time loop on the surrogate's grid with one of its sources,
    `steps` steps after one warm-up step; scenarios/s for 2000-step runs."""
    import oracle  # noqa: F401
    from tests.runners import oracle_model
    os.environ["OMP_NUM_THREADS"] = str(threads)
    base = S.base_grid(0)
    p = S.sample_params(1, 3)[0]
    L = base["xcrd"][-1]
    src = S.source_of(p, L)
    src.pop("rise_time")
    c = dict(base)
    c["H0"] = base["dep"] + S.cg.source_field(c["xcrd"], c["ycrd"], **src)
    m = oracle_model(c)
    m.step(1)
    t0 = time.perf_counter()
    m.step(steps)
    t = (time.perf_counter() - t0) / steps
    return {"value": round(1.0 / (t * 2000), 4), "unit": "scenarios/s", "cores": threads, "kind": "port",
            "steps": steps, "ms_per_step": round(1e3 * t, 3),
            "sample": f"one {S.SIDE}x{S.SIDE} scenario, {steps} time steps after 1 warm-up step, OpenMP over lines "
                      f"({threads} threads), FP64; scenarios/s of 2000-step runs"}


def _json_lines(text):
    out = []
    for ln in text.splitlines():
        ln = ln.strip()
        if ln.startswith("{"):
            try:
                out.append(json.loads(ln))
            except ValueError:
                pass
    return out


def _child(cmd, timeout):
    """Runs one workload in its own process (its own CUDA context: a failure
    there leaves this process's line intact); returns its JSON lines, or an
    error string."""
    t0 = time.perf_counter()
    try:
        p = subprocess.run([sys.executable, *cmd], cwd=ROOT, capture_output=True, text=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return None, f"timed out after {timeout} s", time.perf_counter() - t0
    lines = _json_lines(p.stdout)
    if p.returncode != 0 or not lines:
        tail = (p.stderr or p.stdout).strip().splitlines()[-1:] or [""]
        return None, f"exit {p.returncode}: {tail[0][:200]}", time.perf_counter() - t0
    return lines, None, time.perf_counter() - t0


def side_workloads():
    """The other configurations of the benchmark set, each run whole in its
    own process after the main line's measurements and summarised into it:
    the batched ensemble of 256 scenarios (200 timed steps against the same
    scenarios one at a time), the learned surrogate (4096 training runs from
    the batched solver, networks trained on the GPU, gated passes over 256
    held-out scenarios against one-at-a-time solves) and the nested spherical
    chain (4320 x 2160 master, 600^2 and 900^2 children, 6 model hours)."""
    res = {}
    lines, err, wall = _child(["bench.py", "--workload", "ensemble256", "--steps", "200", "--warmup", "5"], 900)
    if err:
        res["ensemble256"] = {"error": err}
    else:
        e = lines[-1]
        res["ensemble256"] = {
            "command": "python bench.py --workload ensemble256 --steps 200 --warmup 5",
            "metric": e["metric"], "value": e["value"], "unit": e["unit"], "ms_per_step": e["ms_per_step"],
            "one_at_a_time": e["sequential"], "speedup_vs_one_at_a_time": e["speedup_vs_sequential"],
            "plan": e["config"].get("plan"), "autotune_ms_per_step": e["autotune_ms_per_step"],
            "e2e": e["e2e"], "hbm_frac_step": e["roofline"]["frac"],
            "cpu_baseline": e["cpu_baseline"], "gpu_launches": e["gpu_launches"], "wall_s": round(wall, 1)}
    lines, err, wall = _child(["bench.py", "--workload", "surrogate", "--steps", "3", "--warmup", "1"], 1200)
    if err:
        res["surrogate"] = {"error": err}
    else:
        s = lines[-1]
        res["surrogate"] = {
            "command": "python bench.py --workload surrogate --steps 3 --warmup 1",
            "metric": s["metric"], "value": s["value"], "unit": s["unit"],
            "one_at_a_time_scenarios_per_s": s["one_at_a_time_scenarios_per_s"],
            "speedup_vs_one_at_a_time": s["speedup_vs_one_at_a_time"],
            "gauge_rel_err_gated_mean": s["gauge_rel_err_gated_mean"], "fallback": s["fallback"],
            "map_iou_mean": s["map_iou_mean"], "infer_scenarios_per_s": s["infer_scenarios_per_s"],
            "data_seconds": s["data_seconds"], "train_seconds": s["train_seconds"],
            "roofline": s["roofline"], "wall_s": round(wall, 1)}
    lines, err, wall = _child(["cliffs-src_gb300/nested.py", "--scale", "full", "--hours", "6"], 900)
    if err:
        res["nested_sphere"] = {"error": err}
    else:
        tot = lines[-1]
        res["nested_sphere"] = {
            "command": "python cliffs-src_gb300/nested.py --scale full --hours 6",
            "levels": [{k: lv.get(k) for k in ("name", "shape", "t0", "steps", "wall_s", "cell_updates_per_s",
                                               "status", "max_eta", "land_wetted") if k in lv} for lv in lines[:-1]],
            "wall_s": tot["wall_s"], "cell_updates": tot["cell_updates"],
            "mcell_updates_per_s": round(tot["cell_updates_per_s"] / 1e6, 1)}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kernels-only", action="store_true")
    ap.add_argument("--workload", default="shelf2048", choices=["shelf2048", "sphere4320", "ensemble256", "surrogate"])
    ap.add_argument("--sweep", default="tiled", choices=["tiled", "direct", "staged"],
                    help="sweep kernels of the device-resident passes (cliffs_gpu_set_sweep_kernel)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.warmup + args.steps > HORIZON:
        args.warmup = min(args.warmup, 100)
        args.steps = HORIZON - args.warmup
    if args.workload == "ensemble256":
        return run_ensemble(args)
    if args.workload == "surrogate":
        return run_surrogate(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
