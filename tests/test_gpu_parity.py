"""GPU parity against the FP64 oracle, through the C ABI.

Tolerances (the stated parity bar, FP32 state): eta and max-wave elevation within
1e-4 of the source amplitude on cells wet in both runs; velocities within
2e-4 m/s + 2e-4 relative; wet/dry mismatches counted and bounded; gauges
within 1e-4 of the amplitude.  The GPU keeps the state as FP32 surface
elevation; the oracle keeps FP64 celerity exactly as the reference does.
"""
import importlib
import json

import numpy as np
import pytest

import oracle
from tests.lines import random_grid, random_spacing
from tests.runners import (GRAV, compare_maxwave, compare_runup, compare_state, gpu_grid, maxwave_ties,
                           oracle_model, shadow)

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads


def _line_models(rng, n, nlines, iu, ground=0.01, crough=0.002):
    dep, cel, u, v = random_grid(rng, nlines, n, ground=ground, exact_thresholds=False)
    if iu == 2:
        dep, cel, u, v = (np.ascontiguousarray(a.T) for a in (dep, cel, u, v))
    ny, nx = dep.shape
    dx = random_spacing(rng, nx)
    dy = random_spacing(rng, ny)
    zeta = rng.uniform(-2e-8, 2e-8, ny)
    m = oracle.Model(dep, np.tile(dx, (ny, 1)), dy, zeta, ground=ground, crough=crough, dt=0.05)
    m.cel[...] = cel
    m.xvel[...] = u
    m.yvel[...] = v
    e1 = rng.uniform(-0.3, 0.3, (3, m.mx))
    e2 = rng.uniform(-0.3, 0.3, (3, m.mx))
    m.edge1[...] = e1
    m.edge2[...] = e2
    g = pkg.GpuGrid(dep, dx=dx, dy=dy, zeta=zeta, ground=ground, crough=crough, dt=0.05)
    g.upload_state(cel, u, v)
    g.set_edges(e1, e2)
    return m, g


@pytest.mark.parametrize("iu", [1, 2])
@pytest.mark.parametrize("n", [3, 5, 17, 64, 200])
def test_single_sweep_adversarial_lines(iu, n):
    """One sweep over lines that hit every wet/dry branch (cliffs.f:56-329)."""
    rng = np.random.default_rng(100 * iu + n)
    m, g = _line_models(rng, n, 300, iu)
    m.sweep(iu)
    g.sweep(iu)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, 1.0)
    assert r["mismatch"] <= 2, r
    assert r["eta"] <= 2e-5, r          # m, values up to ~2 m
    wet = (m.cel > m.celmin) & (cel > m.celmin)
    du = np.abs(m.xvel - u)[wet]
    dv = np.abs(m.yvel - v)[wet]
    assert (du <= 2e-4 + 2e-4 * np.abs(m.xvel[wet])).all(), du.max()
    assert (dv <= 2e-4 + 2e-4 * np.abs(m.yvel[wet])).all(), dv.max()
    g.close()


def test_fully_dry_lines_untouched():
    """cliffs.f:113: a line without a wet cell is left exactly as it was."""
    rng = np.random.default_rng(9)
    m, g = _line_models(rng, 40, 64, 1)
    cel = np.full_like(m.cel, 0.5 * m.celmin)  # dry, with residual celerity
    g.upload_state(cel, m.xvel, m.yvel)
    before = g.download_state()
    g.sweep(1)
    after = g.download_state()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    g.close()


def test_channel_1d_runup():
    """1-D channel, solitary wave running up a 1:20 beach, 5000 steps."""
    case = W.channel_1d(seed=11)
    A = case["amplitude"]
    m = oracle_model(case)
    g = gpu_grid(case)
    for blk in range(10):
        m.step(500)
        done, _ = g.step(500)
        assert done == 500
        cel, u, v = g.download_state()
        r = compare_state(m, cel, u, v, A)
        assert r["mismatch"] <= 2, (blk, r)
        assert r["eta"] <= 1e-4, (blk, r)
        assert r["u"] <= 2e-4, (blk, r)
    mo, vo = m.maxwave()
    mg, vg = g.maxwave()
    rm = compare_maxwave(mo, vo, mg, vg, A, maxwave_ties(m))
    assert rm["mismatch"] <= 2 and rm["maxe"] <= 1e-4, rm
    # runup: the highest land elevation reached, and the runup line (the
    # landward-most node ever wet) of the oracle exactly
    ro = g.runup()
    land = (m.dep < 0) & (m.hmax > m.celmin)
    ref_runup = float((-m.dep[land]).max()) if land.any() else 0.0
    assert ro["max_runup"] == ref_runup, (ro, ref_runup)
    ru = compare_runup(mo, mg, case["dep"])
    assert ru["rows_differ"] == 0 and ru["runup_gpu_m"] == ref_runup, ru
    assert ro["wetted_land"] > 0
    assert g.status() == (0, 0)
    g.close()


@pytest.mark.parametrize("seed", [13, 17])
def test_channel_1d_runup_front_departure(seed):
    """Seeds whose run-up passes a near-tie of the wet/dry switch (a flooded
    cell ending a step within ~1e-4 m of ground, cliffs.f:56-122).  The free
    FP32 run then departs from the FP64 oracle at the runup front.  The test
    names the step and cell where the free-run eta difference first exceeds
    1e-4 of the amplitude and checks that the cell is in the swash zone (a
    thin water column over the beach), reports the free-run divergence at the
    end beside the windowed comparison (250-step windows restarted from the
    GPU's state, each within 1e-4 of the amplitude), and checks that the
    runup line, the max runup and the wet/dry state still match the oracle's
    exactly."""
    case = W.channel_1d(seed=seed)
    A = case["amplitude"]
    m = oracle_model(case)
    g = gpu_grid(case)
    first = None
    for s in range(1, 5001):
        m.step(1)
        g.step(1)
        if first is None:
            cel, u, v = g.download_state()
            wet = (m.cel > m.celmin) & (cel > m.celmin)
            eo = m.cel ** 2 / GRAV - m.dep
            eg = cel * np.abs(cel) / GRAV - m.dep
            err = np.where(wet, np.abs(eo - eg), 0.0)[0]
            if err.max() > 1e-4 * A:
                k = int(np.argmax(err))
                first = dict(step=s, cell=k + 1, dep=float(m.dep[0, k]), H=float(m.cel[0, k] ** 2 / GRAV),
                             err=float(err[k] / A))
    cel, u, v = g.download_state()
    free = compare_state(m, cel, u, v, A)
    mo, vo = m.maxwave()
    mg, vg = g.maxwave()
    ru = compare_runup(mo, mg, case["dep"])
    g.close()
    # the same case compared over windows restarted from the GPU's state
    m2, g2 = oracle_model(case), gpu_grid(case)
    windows = shadow(m2, g2, 5000, 250, A)
    g2.close()
    print(json.dumps(dict(seed=seed, first_departure=first, free_run_end=free,
                          windowed_worst=max(w["eta"] for w in windows), runup=ru)))
    assert first is not None  # this seed does part from the oracle
    assert first["H"] < 0.1 and first["dep"] < 0.2, first  # in the swash zone of the 1:20 beach
    assert max(w["eta"] for w in windows) <= 1e-4, windows
    assert max(w["mismatch"] for w in windows) == 0, windows
    assert free["mismatch"] == 0, free
    assert ru["rows_differ"] == 0 and ru["runup_gpu_m"] == ru["runup_oracle_m"], ru


@pytest.mark.parametrize("nx,ny,steps", [(256, 256, 600), (320, 200, 300)])
def test_shelf_2d(nx, ny, steps):
    """2-D shelf/slope basin with an elliptical uplift, friction on."""
    case = W.shelf_2d(seed=nx + ny, nx=nx, ny=ny, dx=100.0 * 2048 / nx, steps=steps, ngauges=32)
    case["crough"] = 0.000625
    A = case["amplitude"]
    m = oracle_model(case)
    g = gpu_grid(case)
    I, J = case["gauges"]
    for blk in range(3):
        m.step(steps // 3)
        g.step(steps // 3)
        ge, gu, gv = g.gauges(I, J)
        oe, ou, ov = m.gauges(I, J)
        assert np.abs(ge - oe).max() <= 1e-4 * A
        assert np.abs(gu - ou).max() <= 2e-4
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, A)
    assert r["mismatch"] <= nx * ny // 20000 + 2, r
    assert r["eta"] <= 1e-4, r
    assert r["u"] <= 2e-4 and r["v"] <= 2e-4, r
    mo, vo = m.maxwave()
    mg, vg = g.maxwave()
    rm = compare_maxwave(mo, vo, mg, vg, A, maxwave_ties(m))
    assert rm["mismatch"] <= nx * ny // 20000 + 2 and rm["maxe"] <= 1e-4, rm
    # screenshots (output_sea_state.f)
    ho, uo, _ = m.sea_state(3, 2)
    hg, ug, _ = g.sea_state(3, 2)
    both = (ho > -1e30) & (hg > -1e30)
    assert np.abs(ho - hg)[both].max() <= 1e-4 * A
    g.close()


def test_full_size_2048_short():
    """The benchmark grid itself (2048^2, 100 m), first 40 steps vs oracle."""
    case = W.shelf_2d(seed=0, nx=2048, ny=2048, dx=100.0, steps=40, ngauges=64)
    A = case["amplitude"]
    m = oracle_model(case)
    g = gpu_grid(case)
    m.step(40)
    g.step(40)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, A)
    assert r["mismatch"] <= 20, r
    assert r["eta"] <= 1e-4, r
    g.close()


def test_lake_at_rest_2048():
    """Still water over rough bathymetry with land stays still (well-balanced)."""
    case = W.shelf_2d(seed=5, nx=2048, ny=2048, dx=100.0, steps=200, amp=0.0, ngauges=0)
    g = gpu_grid(case)
    g.step(200)
    cel, u, v = g.download_state()
    wet = cel > g.celmin
    eta = cel * np.abs(cel) / GRAV - case["dep"]
    assert np.abs(eta[wet]).max() < 1e-4
    assert np.abs(u[wet]).max() < 1e-5 and np.abs(v[wet]).max() < 1e-5
    g.close()


def test_deterministic():
    case = W.shelf_2d(seed=2, nx=512, ny=384, dx=400.0, steps=50, ngauges=0)
    a = gpu_grid(case)
    b = gpu_grid(case)
    a.step(50)
    b.step(50)
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    a.close()
    b.close()
