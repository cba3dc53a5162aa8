"""A nested chain on the GPU (nested.run_chain) against the same chain replayed
on the oracle: a spherical master and two children at refinement 3, each fed
by its parent's edge records (feed_children_grid.f, get_boundary_feed.f),
runup on the innermost level and walls on the others.

The chain is the benchmark's nested configuration at a tenth of the size
(nested.SMALL: a 432 x 216 master at 1/12 degree, children of 60^2 and 90^2,
a +3/-1 m dipole source 400 km offshore), for the configuration's full 6
hours of model time.  Every level is compared on its own: the start time and
record count, the gauge series, the max-wave fields and the runup line (per
row, the landward-most node ever wet; on the innermost level the wave runs
up onto land).  Tolerances are those of test_gpu_parity.py: elevation 1e-4
of the source amplitude, velocities 2e-4 m/s; the runup line must be the
oracle's in every row.
"""
import importlib

import numpy as np
import pytest

import oracle
from tests.runners import compare_runup

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
nested = importlib.import_module("cliffs-src_gb300.nested")
cg = pkg.cliffs_gpu

HOURS = 6.0
CUKE = 0.001
BNDOUT, GOUT = 3, 10
A = 3.0


def _oracle_chain(levels, source):
    """run_chain restated on the oracle: the same setup (rest, bottom
    deformation, feed start), the same record and gauge times."""
    t_end = HOURS * 3600.0
    src = {k: v for k, v in source.items() if k != "bottom"}
    out, feed = [], None
    for k, c in enumerate(levels):
        f = int(round(levels[0]["dt"] / c["dt"]))
        bnd, gout = BNDOUT * f, GOUT * f
        child = levels[k + 1] if k + 1 < len(levels) else None
        s1, s2, zeta = oracle.metrics(c["xcrd"], c["ycrd"], False)
        q = cg.source_field(c["xcrd"], c["ycrd"], **src)
        dep = c["dep"] - q  # cliffs_main.f:205-208: the bottom moves, H stays
        t0, irec = 0.0, 1
        if feed is not None:
            m0 = oracle.Model(dep, s1, s2, zeta, ground=c["ground"], crough=c["crough"], dt=c["dt"])
            m0.set_feed(*feed, irec=1, freeze=True)
            irec = m0.feed_start(CUKE)
            t0 = float(feed[0][irec - 1])
        m = oracle.Model(dep, s1, s2, zeta, ground=c["ground"], crough=c["crough"], dt=c["dt"], cel=c["dep"],
                         t0=t0)
        if feed is not None:
            m.set_feed(*feed, irec=irec, freeze=True)
        tab = oracle.NestTables(c["xcrd"], c["ycrd"], child["xcrd"], child["ycrd"]) if child else None
        I, J = c["gauges"]
        gauges, recs, rt = [], [], []
        arv = False
        total = max(0, int(np.floor((t_end - t0) / c["dt"] + 1e-9)))
        done = 0

        def outputs():
            nonlocal arv
            if tab is not None and done % bnd == 0:
                arv, rec = m.feed_child(tab, CUKE, arv)
                if rec is not None:
                    recs.append(rec)
                    rt.append(m.time)
            if done % gout == 0:
                gauges.append((m.time, m.gauges(I, J)))

        outputs()
        while done < total:
            kk = min(total - done, bnd - done % bnd if tab is not None else gout - done % gout, gout - done % gout)
            got = m.step(kk)
            done += got
            if got < kk:
                break
            outputs()
        out.append(dict(t0=t0, steps=done, gauges=gauges, maxwave=m.maxwave(), records=len(recs)))
        feed = nested._records(recs, rt) if recs else None
    return out


def test_nested_chain_against_oracle():
    levels, source = nested.SMALL()
    got = nested.run_chain(levels, source, HOURS, cuke=CUKE, bndout=BNDOUT, gout=GOUT)
    ref = _oracle_chain(levels, source)
    assert [r["t0"] for r in got][0] == 0.0 and got[1]["t0"] > 0 and got[2]["t0"] > got[1]["t0"]
    for k, (g, o) in enumerate(zip(got, ref)):
        assert g["status"] == 0, (k, g["flags"])
        assert abs(g["t0"] - o["t0"]) < 1e-9, k
        assert g["steps"] == o["steps"] and g["records_out"] == o["records"], k
        # gauges (output_gages.f): same record times, eta/u/v
        assert len(g["gauges"]["t"]) == len(o["gauges"]), k
        for r, (t, (eo, uo, vo)) in enumerate(o["gauges"]):
            assert abs(g["gauges"]["t"][r] - t) < 1e-6, (k, r)
            both = np.isfinite(eo) & np.isfinite(g["gauges"]["eta"][r])
            assert (np.isfinite(eo) == np.isfinite(g["gauges"]["eta"][r])).all(), (k, r)
            assert np.abs(g["gauges"]["eta"][r] - eo)[both].max(initial=0.0) <= 1e-4 * A, (k, r)
            assert np.abs(g["gauges"]["u"][r] - uo).max() <= 2e-4, (k, r)
            assert np.abs(g["gauges"]["v"][r] - vo).max() <= 2e-4, (k, r)
        # max-wave fields (output_maxwave.f)
        mo, vo = o["maxwave"]
        so, sg = mo > -1e30, g["maxe"] > -1e30
        assert (so != sg).sum() <= 4, k
        both = so & sg
        assert np.abs(g["maxe"] - mo)[both].max() <= 1e-4 * A, k
        assert np.abs(g["maxv"] - vo)[both].max() <= 2e-4, k
        ru = compare_runup(mo, g["maxe"], levels[k]["dep"])
        assert ru["rows_differ"] == 0 and ru["runup_gpu_m"] == ru["runup_oracle_m"], (k, ru)
    # the wave ran up on the innermost grid: land cells (dep < 0) got wet
    land_wet = (levels[2]["dep"] < 0) & (got[2]["maxe"] > -1e30)
    assert land_wet.sum() > 0
    assert np.abs(got[0]["maxe"][got[0]["maxe"] > -1e30]).max() > 0.5  # the source's wave, not a state at rest
