"""GPU parity of the time loop's other pieces, through the C ABI:

- boundary forcing: start record (get_boundary_feed.f:144-167), record cursor,
  FP64 lerp and the freeze stop (cliffs_main.f:305-339);
- nested-grid feed: arrival test and edge records (feed_children_grid.f);
- spherical grids: cos(lat) row factor and the zeta metric term (MasterGrid.f);
- 1-D channels along y with a width term (MasterGrid.f:118-121);
- 1-D grids with a passive second row;
- non-finite state reported through the status word.
Tolerances as in test_gpu_parity.py.
"""
import importlib

import numpy as np
import pytest

import oracle
from tests.runners import GRAV, compare_maxwave, compare_state, maxwave_ties, shadow

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads


def _pair(case):
    s1, s2, zeta = oracle.metrics(case["xcrd"], case["ycrd"], case["cartesian"])
    if case.get("zeta") is not None:
        zeta = case["zeta"]
    m = oracle.Model(case["dep"], s1, s2, zeta, ground=case["ground"], crough=case["crough"],
                     dt=case["dt"], cel=case["H0"], xvel=case.get("u0"), yvel=case.get("v0"),
                     t0=case.get("t0", 0.0))
    g = pkg.GpuGrid.from_case(case)
    return m, g


def _records(nt, length, t, amp, phase):
    """(nt, 3, length) records: u, v, eta of a sinusoidal wave."""
    r = np.zeros((nt, 3, length))
    s = np.linspace(0, 1, length)
    for k in range(nt):
        w = amp * np.sin(2 * np.pi * (t[k] / 200.0 + phase)) * (0.5 + 0.5 * np.cos(np.pi * s))
        r[k, 2] = w
        r[k, 0] = 0.3 * w
        r[k, 1] = 0.05 * w
    return r


@pytest.mark.parametrize("freeze", [True, False])
def test_boundary_forcing(freeze):
    case = W.shelf_2d(seed=21, nx=160, ny=120, dx=1000.0, steps=0, amp=0.0, ngauges=8,
                      perturb=0.02)
    ny, nx = case["dep"].shape
    nt = 30
    rec_dt = 8 * case["dt"]
    tin = np.arange(nt) * rec_dt
    west = _records(nt, ny, tin, 0.4, 0.0)
    east = _records(nt, ny, tin, 0.1, 0.3)
    south = _records(nt, nx, tin, 0.2, 0.1)
    north = _records(nt, nx, tin, 0.05, 0.6)
    west[:3] = 0.0  # a quiet start so the start-record search has work to do
    east[:3] = 0.0
    south[:3] = 0.0
    north[:3] = 0.0
    m, g = _pair(case)
    m.set_feed(tin, west, east, south, north, irec=1, freeze=freeze)
    cuke = 0.01
    irec = m.feed_start(cuke)
    g.set_feed(tin, west, east, south, north, irec=1, freeze=freeze)
    assert g.feed_start(cuke) == irec and irec > 1
    m.set_feed(tin, west, east, south, north, irec=irec, freeze=freeze)
    g.set_feed(tin, west, east, south, north, irec=irec, freeze=freeze)
    m.t.value = tin[irec - 1]
    g.t.value = tin[irec - 1]
    total = int((tin[-1] - tin[irec - 1]) / case["dt"]) + 40  # runs past the last record
    done_o = m.step(total)
    done_g, ended = g.step(total)
    assert done_g == done_o
    assert ended == freeze and (done_o < total) == freeze
    assert abs(g.time - m.time) < 1e-9
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, 0.4)
    assert r["mismatch"] <= 2, r
    assert r["eta"] <= 1e-4, r
    assert r["u"] <= 2e-4 and r["v"] <= 2e-4, r
    mo, vo = m.maxwave()
    mg, vg = g.maxwave()
    rm = compare_maxwave(mo, vo, mg, vg, 0.4, maxwave_ties(m))
    assert rm["mismatch"] <= 2 and rm["maxe"] <= 1e-4, rm
    g.close()


def test_nested_feed_records():
    case = W.shelf_2d(seed=31, nx=256, ny=200, dx=800.0, steps=0, ngauges=0,
                      centre_km=(120.0, 80.0))
    m, g = _pair(case)
    x, y = case["xcrd"], case["ycrd"]
    # child at refinement 3 inside the parent, off the grid nodes
    xn = np.arange(x[100] + 133.0, x[180], 800.0 / 3)[:150]
    yn = np.arange(y[40] + 57.0, y[120], 800.0 / 3)[:180]
    tab = oracle.NestTables(x, y, xn, yn)
    nest = g.nest_add(tab.as_dict())
    arr_o = arr_g = False
    seen = 0
    for blk in range(12):
        m.step(20)
        g.step(20)
        arr_o, rec_o = m.feed_child(tab, 0.001, arr_o)
        arr_g, rec_g = g.feed_child(nest, 0.001, arr_g)
        assert arr_o == arr_g, blk
        if rec_o is not None:
            seen += 1
            for ro, rg in zip(rec_o, rec_g):
                assert np.abs(ro[2] - rg[2]).max() <= 1e-4 * case["amplitude"]
                assert np.abs(ro[:2] - rg[:2]).max() <= 2e-4
    assert seen > 3
    g.close()


def test_spherical_grid():
    nx, ny = 240, 200
    lon = np.linspace(140.0, 144.0, nx)
    lat = np.linspace(38.0, 41.5, ny)
    base = W.shelf_2d(seed=41, nx=nx, ny=ny, dx=1500.0, steps=0, ngauges=16)
    case = dict(base, xcrd=lon, ycrd=lat, cartesian=False)
    s1, s2, _ = oracle.metrics(lon, lat, False)
    hmax = float(base["H0"].max())
    case["dt"] = float(0.8 * min(s1.min(), s2.min()) / np.sqrt(GRAV * hmax))
    case["crough"] = 0.000625
    m, g = _pair(case)
    m.step(300)
    g.step(300)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, base["amplitude"])
    assert r["mismatch"] <= 3, r
    assert r["eta"] <= 1e-4, r
    assert r["u"] <= 2e-4 and r["v"] <= 2e-4, r
    I, J = base["gauges"]
    ge, gu, gv = g.gauges(I, J)
    oe, ou, ov = m.gauges(I, J)
    assert np.abs(ge - oe).max() <= 1e-4 * base["amplitude"]
    g.close()


def test_channel_along_y_with_width_term():
    """Run-up and run-down of a large wave in a 1-D channel along y.  The run
    passes near-ties of the wet/dry switch (tests/test_oracle_conditioning.py),
    so it is compared over 250-step windows restarted from the GPU state."""
    c1 = W.channel_1d(seed=5, n=1200, steps=0)
    ny = c1["dep"].shape[1]
    yc = c1["xcrd"]
    # the channel runs along y (nx = 1); zeta carries the width variation
    width = 1.0 + 0.3 * np.tanh((yc - 30.0) / 10.0)
    zeta = np.gradient(width, yc) / width / 8.0
    case = dict(c1, xcrd=np.zeros(1), ycrd=yc, dep=c1["dep"].reshape(ny, 1),
                H0=c1["H0"].reshape(ny, 1), u0=np.zeros((ny, 1)), v0=np.zeros((ny, 1)), zeta=zeta)
    m, g = _pair(case)
    for k, r in enumerate(shadow(m, g, 2500, 250, c1["amplitude"])):
        assert r["mismatch"] <= 2, (k, r)
        assert r["eta"] <= 1e-4, (k, r)
        assert r["v"] <= 2e-4, (k, r)
    g.close()


def test_one_d_with_passive_row():
    c1 = W.channel_1d(seed=8, n=800, steps=0)
    n = c1["dep"].shape[1]
    dep = np.vstack([c1["dep"], c1["dep"] - 0.25])
    H0 = np.vstack([c1["H0"], c1["dep"] - 0.25])
    case = dict(c1, ycrd=np.array([0.0, 1.0]), dep=dep.astype(np.float32).astype(np.float64),
                H0=H0, u0=np.zeros((2, n)), v0=np.zeros((2, n)))
    m, g = _pair(case)
    m.step(1500)
    g.step(1500)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, c1["amplitude"])
    assert r["mismatch"] <= 2 and r["eta"] <= 1e-4, r
    g.close()


def test_nonfinite_state_is_reported():
    case = W.shelf_2d(seed=2, nx=128, ny=96, dx=1000.0, steps=0, ngauges=0)
    g = pkg.GpuGrid.from_case(case)
    cel, u, v = g.download_state()
    u[40, 50] = np.nan
    g.upload_state(cel, u, v)
    g.step(2)
    r, flags = g.status()
    assert r == pkg.cliffs_gpu.CliffsError(-3, "x").code and flags & 1
    r, flags = g.status()  # the status word is cleared by reading it
    assert flags == 0
    g.close()


def test_courant_check():
    """A time step past the Courant limit is reported (CLIFFS_ST_CFL, status
    CLIFFS_WARN_CFL) with the largest Courant number the sweeps read; the
    workload's own time step (Courant 0.8 on the deepest water) raises
    nothing."""
    case = W.shelf_2d(seed=4, nx=256, ny=192, dx=1000.0, steps=0, ngauges=0)
    g = pkg.GpuGrid.from_case(case)
    g.step(20)
    assert g.status() == (0, 0)
    assert g.courant() == 0.0
    g.close()
    case["dt"] *= 1.5
    g = pkg.GpuGrid.from_case(case)
    g.step(1)
    r, flags = g.status()
    assert r == pkg.cliffs_gpu.CLIFFS_WARN_CFL and flags == pkg.cliffs_gpu.CLIFFS_ST_CFL, (r, flags)
    # the first x-sweep reads the state at rest: sqrt(g H) dt / dx at the
    # deepest cell (H in FP32 as the device holds it)
    H = np.asarray(case["H0"], np.float32).astype(np.float64)
    expect = np.sqrt(GRAV * H.max()) * case["dt"] / 1000.0
    cn = g.courant()
    assert expect * (1 - 1e-4) <= cn <= expect * 1.05, (cn, expect)
    assert g.status() == (0, 0)  # read and cleared
    assert g.courant() == cn     # the largest number stays reported
    g.close()
