"""The headline configurations for their full length, free-running, against
the FP64 oracle, through the C ABI.

- The 2048^2 Cartesian shelf for all 3000 steps of its configuration: the 64
  gauges every 10 steps, the final state, the max-wave fields, the wet/dry
  mismatch count and the runup line.
- The 4320 x 2160 spherical grid for 600 steps (the same checks).

Tolerances are those of test_gpu_parity.py (eta, max-wave and gauges within
1e-4 of the source amplitude, velocities within 2e-4 m/s); the wet/dry
mismatch count must be 0, and the runup line (per row, the landward-most
node ever wet, output_maxwave.f:14-27 / cliffs.f:56-122) must be the
oracle's in every row.  Each test prints its report (pytest -s shows it).
The oracle runs with OpenMP on every host core: ~80 s for the shelf.
"""
import importlib
import json

import numpy as np
import pytest

from tests.runners import compare_maxwave, compare_runup, compare_state, gpu_grid, maxwave_ties, oracle_model

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads


def _free_run(case, steps, gout=10):
    """Both solvers from the same initial state for `steps` steps, the gauges
    compared every `gout` steps; returns the report."""
    A = case["amplitude"]
    m = oracle_model(case)
    g = gpu_grid(case)
    I, J = case["gauges"]
    worst = dict(eta=0.0, u=0.0, v=0.0, records=0)
    for s in range(gout, steps + 1, gout):
        m.step(gout)
        done, _ = g.step(gout)
        assert done == gout
        eo, uo, vo = m.gauges(I, J)
        eg, ug, vg = g.gauges(I, J)
        wo, wg = eo > -1e30, eg > -1e30
        assert (wo == wg).all(), f"gauge wetness differs at step {s}"
        worst["eta"] = max(worst["eta"], float(np.abs(eg - eo)[wo].max(initial=0.0) / A))
        worst["u"] = max(worst["u"], float(np.abs(ug - uo).max()))
        worst["v"] = max(worst["v"], float(np.abs(vg - vo).max()))
        worst["records"] += 1
    cel, u, v = g.download_state()
    state = compare_state(m, cel, u, v, A)
    mo, vo_ = m.maxwave()
    mg, vg_ = g.maxwave()
    mw = compare_maxwave(mo, vo_, mg, vg_, A, maxwave_ties(m))
    ru = compare_runup(mo, mg, case["dep"])
    status = g.status()
    g.close()
    return dict(gauges=worst, state=state, maxwave=mw, runup=ru, status=status)


def _check(rep):
    print(json.dumps(rep))
    assert rep["status"] == (0, 0), rep["status"]
    gz = rep["gauges"]
    assert gz["eta"] <= 1e-4 and gz["u"] <= 2e-4 and gz["v"] <= 2e-4, gz
    st = rep["state"]
    assert st["mismatch"] == 0, st
    assert st["eta"] <= 1e-4 and st["u"] <= 2e-4 and st["v"] <= 2e-4, st
    mw = rep["maxwave"]
    assert mw["mismatch"] == 0 and mw["maxe"] <= 1e-4 and mw["maxv"] <= 2e-4, mw
    ru = rep["runup"]
    assert ru["rows_differ"] == 0 and ru["one_sided"] == 0, ru
    assert ru["runup_gpu_m"] == ru["runup_oracle_m"], ru


def test_shelf_2048_all_3000_steps():
    case = W.shelf_2d(seed=0, nx=2048, ny=2048, dx=100.0, steps=3000, ngauges=64)
    case["crough"] = 0.000625  # the benchmark's friction
    rep = _free_run(case, 3000)
    _check(rep)
    # the wave reached the coast: the runup line is not the still shoreline
    assert rep["runup"]["runup_oracle_m"] > 1.0, rep["runup"]


def test_sphere_4320x2160_600_steps():
    case = W.sphere_2d(seed=3, nx=4320, ny=2160, steps=600, ngauges=64)
    case["crough"] = 0.000625
    rep = _free_run(case, 600)
    _check(rep)
