"""One-way nested runs (NestedGrid.f, feed_children_grid.f,
get_boundary_feed.f) in one process: a master grid and a chain of children,
every level stepped on the GPU by its own context, the feed between levels
kept in host memory.

The reference runs every level as its own process:
- the parent writes its child's edge records (u, v, eta on the child's four
  edges, bilinear in the parent, dry parent cells as 0) every bndout steps
  once the wave has reached the child's footprint (feed_children_grid.f:10-179,
  output_feed.f);
- the child run reads them back (get_boundary_feed.f:144-167);
- it starts at the first record whose edge elevation reaches cuke
  (get_boundary_feed.f:144-167);
- it interpolates its edge values between records in time
  (cliffs_main.f:305-323) and stops when the records end (freeze).
run_chain does the same without the files: level k runs to the end time and
produces the records of level k+1, which then runs from them.

    python cliffs-src_gb300/nested.py [--scale full|small] [--hours 6]

runs the benchmark's nested configuration (workloads.nested_sphere: a 4320 x
2160 spherical master at 1/12 degree, children of 600^2 and 900^2 at
refinement 3, a +3/-1 m dipole source) and prints one JSON line per level and
a summary.
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


def pinpoint(xx, xp):
    """NestedGrid.f:129-148: the 1-based ip with xx(ip) <= xp <= xx(ip+1)
    (bisection over the ascending xx) and the weight of xx(ip),
    (xx(ip+1) - xp) / (xx(ip+1) - xx(ip))."""
    n = len(xx)
    ip, ipp = 1, n
    while ip + 2 <= ipp:
        med = (ip + ipp) // 2
        if xp > xx[med - 1]:
            ip = med
        else:
            ipp = med
    cp = (xx[ip] - xp) / (xx[ip] - xx[ip - 1]) if n > 1 else 0.5
    return ip, float(cp)


def nest_tables(x, y, xn, yn):
    """The interpolation tables of one child (NestedGrid.f:104-119): the
    parent row and weight of the child's south and north edges and of every
    child row (west/east edges), the parent column and weight of the child's
    west and east edges and of every child column (south/north edges)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    if xn[0] < x[0] or xn[-1] > x[-1] or yn[0] < y[0] or yn[-1] > y[-1]:
        raise ValueError("child grid not within its parent's limits")
    t = {}
    t["S_ny"], t["S_cy"] = pinpoint(y, yn[0])
    t["N_ny"], t["N_cy"] = pinpoint(y, yn[-1])
    t["W_nx"], t["W_cx"] = pinpoint(x, xn[0])
    t["E_nx"], t["E_cx"] = pinpoint(x, xn[-1])
    sn = [pinpoint(x, v) for v in xn]
    we = [pinpoint(y, v) for v in yn]
    t["SN_nx"] = np.array([a for a, _ in sn], np.int32)
    t["SN_cx"] = np.array([b for _, b in sn])
    t["WE_ny"] = np.array([a for a, _ in we], np.int32)
    t["WE_cy"] = np.array([b for _, b in we])
    return t


def _records(recs, times):
    """Feed records in set_feed's layout: tinput (nt), west/east (nt, 3, ny),
    south/north (nt, 3, nx), from a list of (w, e, s, n) records."""
    return (np.asarray(times, np.float64), np.stack([r[0] for r in recs]), np.stack([r[1] for r in recs]),
            np.stack([r[2] for r in recs]), np.stack([r[3] for r in recs]))


def run_level(case, source, t_end, feed=None, child=None, cuke=0.001, bndout=3, gout=10):
    """One level: the grid at rest, the source as a bottom deformation, then
    steps to t_end in chunks of bndout steps.  feed: the records of this level
    (from its parent), child: the next level's case, whose records this level
    produces.  Gauge records every gout steps.  Feed and gauge records are
    asynchronous outputs into pinned host memory, so the loop never waits for
    the device; they are collected at the end.  Returns (result, child_feed)."""
    cg = pkg.cliffs_gpu
    g = pkg.GpuGrid.from_case(case)
    t0 = 0.0
    if feed is not None:
        tin, w, e, s, n = feed
        if len(tin) < 2:
            raise RuntimeError(f"{case['name']}: fewer than 2 feed records")
        g.set_feed(tin, w, e, s, n, irec=1, freeze=True)
        irec = g.feed_start(cuke)
        if irec < 1:
            raise RuntimeError(f"{case['name']}: the feed never reaches cuke")
        g.set_feed(tin, w, e, s, n, irec=irec, freeze=True)
        t0 = float(tin[irec - 1])
        g.t.value = t0
    g.add_source(case["xcrd"], case["ycrd"], **source)
    nest = g.nest_add(nest_tables(case["xcrd"], case["ycrd"], child["xcrd"], child["ycrd"])) if child else None
    total = max(0, int(np.floor((t_end - t0) / case["dt"] + 1e-9)))
    step = bndout if nest is not None else gout
    if step >= 2:
        # the steps between outputs replay from graphs, forced or not
        g.set_graph_steps(min(step, 16))
    I, J = case["gauges"]
    ng = len(I)
    n_g = total // gout + 1
    gbuf = cg.pinned((n_g, 3, ng))
    gt = []
    if nest is not None:
        mm, nn = nest[1]
        n_f = total // bndout + 1
        fbuf = {k: cg.pinned((n_f, 3, m)) for k, m in (("w", nn), ("e", nn), ("s", mm), ("n", mm))}
        farr = cg.pinned((n_f,), np.int32)
        ft = []
    last = -1
    g.sync()
    w0 = time.perf_counter()
    done = 0

    def outputs():
        nonlocal last
        if nest is not None and done % bndout == 0:
            k = len(ft)
            last = g.feed_child_async(nest, cuke, (farr[k:k + 1], fbuf["w"][k], fbuf["e"][k], fbuf["s"][k],
                                                   fbuf["n"][k]))
            ft.append(g.time)
        if done % gout == 0:
            k = len(gt)
            last = g.gauges_async(I, J, (gbuf[k, 0], gbuf[k, 1], gbuf[k, 2]))
            gt.append(g.time)

    outputs()
    ended = False
    while done < total and not ended:
        k = min(total - done, step - done % step, gout - done % gout)
        got, ended = g.step(k)
        done += got
        if got == k:
            outputs()
    me, mv = g.maxwave()  # synchronises: every output above is done after it
    if last >= 0:
        g.wait(last)
    wall = time.perf_counter() - w0
    r, flags = g.status()
    child_feed = None
    if nest is not None:
        got_rec = np.flatnonzero(farr[:len(ft)] == 1)
        if len(got_rec):
            child_feed = (np.asarray(ft)[got_rec], fbuf["w"][got_rec].copy(), fbuf["e"][got_rec].copy(),
                          fbuf["s"][got_rec].copy(), fbuf["n"][got_rec].copy())
    k = len(gt)
    res = dict(name=case["name"], shape=list(case["dep"].shape), dt=case["dt"], t0=t0, t_end=g.time, steps=done,
               feed_ended=bool(ended), wall_s=wall, cell_updates_per_s=case["dep"].size * done / max(wall, 1e-12),
               status=r, flags=flags, launches=g.launches(),
               records_out=0 if child_feed is None else len(child_feed[0]),
               land_wetted=int(((case["dep"] < 0) & (case["dep"] > -900.0) & (me > -1e30)).sum()),
               maxe=me, maxv=mv, gauges=dict(t=np.array(gt), eta=gbuf[:k, 0].copy(), u=gbuf[:k, 1].copy(),
                                             v=gbuf[:k, 2].copy()))
    g.close()
    return res, child_feed


def run_chain(levels, source, hours, cuke=0.001, bndout=3, gout=10):
    """Every level of a nested chain to `hours` of model time, the master
    first.  bndout and gout are in the master's steps; a level of dt/r^k
    counts r^k times as many, so its feed and gauge records fall at the
    master's record times."""
    t_end = hours * 3600.0
    out, feed = [], None
    for k, case in enumerate(levels):
        f = int(round(levels[0]["dt"] / case["dt"]))
        child = levels[k + 1] if k + 1 < len(levels) else None
        res, feed_next = run_level(case, source, t_end, feed=feed, child=child, cuke=cuke, bndout=bndout * f,
                                   gout=gout * f)
        out.append(res)
        if child is not None and feed_next is None:
            raise RuntimeError(f"the wave never reached {child['name']}")
        feed = feed_next
    return out


def SMALL(seed=3):
    """The nested chain at a tenth of the size and the full resolution: a
    432 x 216 master at 1/12 degree (16N-32N), children of 60^2 and 90^2 at
    refinement 3, the source 400 km offshore."""
    return pkg.workloads.nested_sphere(seed=seed, nx=432, ny=216, lat=(16.0, 32.0), dlon=1.0 / 12.0, sizes=(60, 90),
                                       land=4, slope=5, shelf=12, ngauges=8, source_km=400.0)


def summary(res):
    """The scalars of a level's result (no fields)."""
    wet = res["maxe"] > -1e30
    return {k: v for k, v in res.items() if k not in ("maxe", "maxv", "gauges")} | {
        "max_eta": float(res["maxe"][wet].max()) if wet.any() else None,
        "ever_wet_cells": int(wet.sum()), "gauge_records": int(len(res["gauges"]["t"]))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", default="full", choices=["full", "small"])
    ap.add_argument("--hours", type=float, default=6.0)
    ap.add_argument("--seed", type=int, default=3)
    a = ap.parse_args()
    pkg.build.build()
    W = pkg.workloads
    if a.scale == "full":
        levels, source = W.nested_sphere(seed=a.seed)
    else:
        levels, source = SMALL(a.seed)
    w0 = time.perf_counter()
    res = run_chain(levels, source, a.hours)
    wall = time.perf_counter() - w0
    for r in res:
        print(json.dumps(summary(r)), flush=True)
    cells = sum(np.prod(r["shape"]) * r["steps"] for r in res)
    print(json.dumps({"levels": len(res), "hours": a.hours, "wall_s": round(wall, 3),
                      "cell_updates": int(cells), "cell_updates_per_s": cells / wall}), flush=True)


if __name__ == "__main__":
    main()
