"""The C++ driver on the GPU: a whole run from the reference's input files to
its output files, against the oracle replaying the same time loop.

The case (tests/cases.py) has boundary forcing, an initial source with a
bottom deformation, 6 gauges and a nested child grid at refinement 3.  The
driver steps the GPU library from one output event to the next
(cliffs_main.f:300-378) and writes screenshots, gauge records, child feed
records and the max-wave fields; every record is compared with the oracle at
the same step.  Tolerances as in test_gpu_parity.py: elevation 1e-4 of the
source amplitude, velocities 2e-4 m/s.
"""
import importlib
import os
import subprocess

import numpy as np
import pytest
from scipy.io import netcdf_file

import oracle
from tests import cases

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
DRIVER = os.path.join(os.path.dirname(pkg.__file__), "_lib", "cliffs_gb300")
CUKE = 0.001


def _replay(c, ref):
    """cliffs_main.f's event loop on the oracle; returns the records in output order."""
    s1, s2, zeta = oracle.metrics(c["x"], c["y"], True)
    m = oracle.Model(ref["dep"], s1, s2, zeta, ground=c["ground"], crough=c["crough"], dt=c["dt"],
                     cel=ref["H"], xvel=ref["u"], yvel=ref["v"], t0=ref["t0"])
    m.set_feed(c["tinput"], c["west"], c["east"], c["south"], c["north"], irec=ref["irec"],
               freeze=c["freeze"])
    tab = oracle.NestTables(c["x"], c["y"], c["xn"], c["yn"])
    shots, gages, feeds = [], [], []
    state = {"arv": False}

    def sea():
        shots.append((m.time, m.sea_state(c["lonsub"], c["latsub"])))

    def gage():
        gages.append((m.time, m.gauges(c["I"], c["J"])))

    def feed():
        state["arv"], rec = m.feed_child(tab, CUKE, state["arv"])
        if rec is not None:
            feeds.append((m.time, rec))

    sea()
    gage()
    feed()
    total = c["steps"]
    istep = 0
    while istep < total:
        nxt = total
        for every in (c["seaout"], c["gout"], c["maxout"], c["bndout"]):
            nxt = min(nxt, (istep // every + 1) * every)
        done = m.step(nxt - istep)
        istep += done
        if done < nxt - (istep - done):
            break
        if istep % c["bndout"] == 0:
            feed()
        if istep % c["seaout"] == 0:
            sea()
        if istep % c["gout"] == 0:
            gage()
    return shots, gages, feeds, m.maxwave()


def test_driver_run_against_oracle(tmp_path):
    pkg.build.build()
    d = str(tmp_path / "in") + "/"
    c = cases.write_case(d, steps=240, seaout=80, gout=20, maxout=120, bndout=20, amp=1.5)
    ref = cases.reference_setup(c, cuke=CUKE)
    out = str(tmp_path / "out" / "run")
    os.makedirs(os.path.dirname(out))
    r = subprocess.run([DRIVER, out, d, "bnd", "src", d + "params.txt"], capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, (r.stderr, open(out + "_log.txt").read())
    shots, gages, feeds, (mo, vo) = _replay(c, ref)
    A = 1.5
    # screenshots (output_sea_state.f)
    h = netcdf_file(out + "_sea_h.nc", "r", mmap=False)
    u = netcdf_file(out + "_sea_u.nc", "r", mmap=False)
    assert h.variables["ha"].shape[0] == len(shots)
    for k, (t, (ho, uo, _)) in enumerate(shots):
        assert abs(h.variables["time"][k] - t) < 1e-9
        hg = h.variables["ha"][k]
        ug = u.variables["ua"][k]
        both = (ho > -1e30) & (hg > -1e30)
        assert ((ho > -1e30) != (hg > -1e30)).sum() <= 2, k
        assert np.abs(hg - ho)[both].max() <= 1e-4 * A, k
        assert np.abs(ug - uo)[both].max() <= 2e-4, k
    # gauges (output_gages.f)
    g = netcdf_file(out + "_gages.nc", "r", mmap=False)
    assert g.variables["gage"].shape[0] == len(gages)
    for k, (t, (eo, uo, vo_)) in enumerate(gages):
        assert abs(g.variables["time"][k] - t) < 1e-9
        assert np.abs(g.variables["gage"][k] - eo).max() <= 1e-4 * A, k
        assert np.abs(g.variables["u"][k] - uo).max() <= 2e-4, k
        assert np.abs(g.variables["v"][k] - vo_).max() <= 2e-4, k
    # child feed records (feed_children_grid.f via output_feed.f)
    assert len(feeds) > 3
    for side, idx in (("west", 0), ("east", 1), ("south", 2), ("north", 3)):
        f = netcdf_file(out + f"_child_{side}.nc", "r", mmap=False)
        assert f.variables["vals"].shape[0] == len(feeds), side
        for k, (t, rec) in enumerate(feeds):
            assert abs(f.variables["time"][k] - t) < 1e-9
            vg = f.variables["vals"][k]
            assert np.abs(vg[2] - rec[idx][2]).max() <= 1e-4 * A, (side, k)
            assert np.abs(vg[:2] - rec[idx][:2]).max() <= 2e-4, (side, k)
    # max-wave fields at the end (output_maxwave.f)
    mx = netcdf_file(out + "_maxwave.nc", "r", mmap=False)
    mg, vg = mx.variables["MaxE"][:], mx.variables["MaxV"][:]
    both = (mo > -1e30) & (mg > -1e30)
    assert ((mo > -1e30) != (mg > -1e30)).sum() <= 4
    assert np.abs(mg - mo)[both].max() <= 1e-4 * A
    assert np.abs(vg - vo)[both].max() <= 2e-4
    log = open(out + "_log.txt").read()
    assert "reached child grid 1" in log and "time loop" in log
