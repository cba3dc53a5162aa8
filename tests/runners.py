"""Shared helpers: run one case on the GPU library and on the oracle, compare."""
import importlib

import numpy as np

import oracle

pkg = importlib.import_module("cliffs-src_gb300")
GRAV = oracle.GRAV


def oracle_model(case):
    s1, s2, zeta = oracle.metrics(case["xcrd"], case["ycrd"], case["cartesian"])
    if case.get("zeta") is not None:
        zeta = case["zeta"]
    return oracle.Model(case["dep"], s1, s2, zeta, ground=case["ground"], crough=case["crough"],
                        dt=case["dt"], cel=case["H0"], xvel=case.get("u0"), yvel=case.get("v0"),
                        t0=case.get("t0", 0.0))


def oracle_model32(case):
    """The FP32 variant of the oracle's time loop on a case (a timed baseline)."""
    s1, s2, zeta = oracle.metrics(case["xcrd"], case["ycrd"], case["cartesian"])
    if case.get("zeta") is not None:
        zeta = case["zeta"]
    return oracle.Model32(case["dep"], s1, s2, zeta, ground=case["ground"], crough=case["crough"], dt=case["dt"],
                          cel=case["H0"], xvel=case.get("u0"), yvel=case.get("v0"))


def gpu_grid(case):
    return pkg.GpuGrid.from_case(case)


def compare_state(m, cel, u, v, scale):
    """Differences between oracle model m and a GPU state (cel, u, v).

    Returns a dict: wet/dry mismatch count and the max |difference| of eta, u,
    v over cells wet in both, eta relative to `scale`.
    """
    wo = m.cel > m.celmin
    wg = cel > m.celmin
    both = wo & wg
    eo = m.cel ** 2 / GRAV - m.dep
    eg = cel * np.abs(cel) / GRAV - m.dep
    # a flooded cell that is not updated holds exactly celmin in the oracle;
    # the FP32 path lands within an ulp either side: a tie, not a mismatch
    tie = np.abs(m.cel - m.celmin) <= 1e-5 * m.celmin
    diff = wo != wg
    res = dict(mismatch=int((diff & ~tie).sum()), ties=int((diff & tie).sum()), wet=int(wo.sum()))
    if both.any():
        res["eta"] = float(np.abs(eo - eg)[both].max() / scale)
        res["u"] = float(np.abs(m.xvel - u)[both].max())
        res["v"] = float(np.abs(m.yvel - v)[both].max())
    else:
        res["eta"] = res["u"] = res["v"] = 0.0
    return res


def compare_maxwave(mo, vo, mg, vg, scale, tie_mask=None):
    so = mo > -1e30
    sg = mg > -1e30
    both = so & sg
    r = dict(mismatch=int((so != sg).sum()))
    # cells whose maximum was a flooded cell at exactly celmin are ties
    if tie_mask is not None:
        r["mismatch"] = int(((so != sg) & ~tie_mask).sum())
    r["maxe"] = float(np.abs(mo - mg)[both].max() / scale) if both.any() else 0.0
    r["maxv"] = float(np.abs(vo - vg)[both].max()) if both.any() else 0.0
    return r


def maxwave_ties(m):
    """Cells whose oracle hmax sits exactly at celmin (see compare_state)."""
    return np.abs(m.hmax - m.celmin) <= 1e-5 * m.celmin


def restart_from(m, cel, u, v):
    """Put a GPU state (the celerity form of download_state) into oracle m."""
    m.cel[...] = cel
    m.xvel[...] = u
    m.yvel[...] = v


def shadow(m, g, steps, window, scale):
    """Run oracle m and GPU grid g side by side for `steps` steps, restarting
    the oracle from the GPU state at the start of every `window` steps.

    The wet/dry switch of the reference scheme (a cell is land when its depth
    is <= ground, cliffs.f:60-70) is discontinuous: a run-down that leaves a
    newly flooded cell within ~1e-5 of `ground` takes one branch or the other
    depending on rounding, and the branch taken moves the rest of the run by up
    to ~1e-2 of the amplitude (test_oracle_conditioning pins this on the
    oracle alone).  Free-running FP32 and FP64 runs of such a case part at the
    first such near-tie, so the scheme is compared over windows: from the same
    state, `window` steps of the GPU must agree with `window` steps of the
    oracle.  Returns the per-window compare_state reports.
    """
    out = []
    done = 0
    while done < steps:
        k = min(window, steps - done)
        cel, u, v = g.download_state()
        restart_from(m, cel, u, v)
        m.step(k)
        got, _ = g.step(k)
        assert got == k
        done += k
        cel, u, v = g.download_state()
        out.append(compare_state(m, cel, u, v, scale))
    return out


def runup_line(maxe):
    """Per row of a max-wave elevation field (output_maxwave.f:14-27, -1e32
    where never wet): the landward-most node ever wet, i.e. the largest x
    index with hmax > celmin (the coast of every workload lies on the high-x
    side); -1 for a row never wet."""
    wet = maxe > -1e30
    last = wet.shape[1] - 1 - np.argmax(wet[:, ::-1], axis=1)
    return np.where(wet.any(axis=1), last, -1)


def compare_runup(mo, mg, dep):
    """The runup line of the GPU's max-wave field mg against the oracle's mo:
    per row, the landward-most wetted node, GPU minus oracle, in cells and in
    metres of ground elevation (-dep) at those nodes.  Also the runup itself,
    the highest land elevation (-dep over dep < 0) ever wetted, of each."""
    io, ig = runup_line(mo), runup_line(mg)
    rows = np.nonzero((io >= 0) | (ig >= 0))[0]
    r = dict(rows=int(len(rows)), rows_differ=0, max_cells=0, max_elev_m=0.0)
    if len(rows):
        both = rows[(io[rows] >= 0) & (ig[rows] >= 0)]
        dc = ig[both] - io[both]
        de = np.abs(dep[both, ig[both]] - dep[both, io[both]])
        r["rows_differ"] = int((io[rows] != ig[rows]).sum())
        r["max_cells"] = int(np.abs(dc).max()) if len(dc) else 0
        r["max_elev_m"] = float(de.max()) if len(de) else 0.0
        r["one_sided"] = int(len(rows) - len(both))
        if r["rows_differ"]:
            k = rows[np.argmax(np.abs(np.where(io[rows] >= 0, io[rows], 0) - np.where(ig[rows] >= 0, ig[rows], 0)))]
            r["worst_row"] = dict(j=int(k) + 1, i_oracle=int(io[k]) + 1, i_gpu=int(ig[k]) + 1)
    for key, m in (("runup_oracle_m", mo), ("runup_gpu_m", mg)):
        land = (dep < 0) & (m > -1e30)
        r[key] = float((-dep[land]).max()) if land.any() else 0.0
    return r
