"""Analytic sources on the device (cliffs_gpu_add_source) against the
reference's setup restated on the oracle.

- surface deformation (cliffs_main.f:209-213): H = dep + q, then the
  celerity transform;
- bottom deformation (cliffs_main.f:205-208, quake = 1): the bottom moves by
  -q under the water column at rest;
- a surface uplift rising linearly over a rise time, which the oracle run
  receives as the same increments before each step.
The uplift field itself is compared with numpy's FP64 evaluation of the
formula (cliffs_gpu.source_field).
"""
import importlib

import numpy as np
import pytest

from tests.runners import GRAV, compare_state, oracle_model

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
cg = pkg.cliffs_gpu
W = pkg.workloads

SRC = dict(x0=9000.0, y0=7000.0, ax=4000.0, ay=2000.0, angle=0.6, amp=1.2, dipole=0.4)


def _case(seed=71):
    c = W.shelf_2d(seed=seed, nx=200, ny=160, dx=100.0, steps=0, amp=0.0, ngauges=0)
    c["crough"] = 0.000625
    c["H0"] = c["dep"].copy()
    return c


def _oracle(c, dep, H):
    case = dict(c, dep=dep, H0=H)
    return oracle_model(case)


def _transform(H, ground):
    return np.where(H > ground, H, 0.0)


@pytest.mark.parametrize("bottom", [False, True])
def test_instant_source_against_oracle(bottom):
    c = _case()
    q = cg.source_field(c["xcrd"], c["ycrd"], **SRC)
    g = pkg.GpuGrid.from_case(c)
    g.add_source(c["xcrd"], c["ycrd"], bottom=bottom, **SRC)
    if bottom:
        m = _oracle(c, c["dep"] - q, c["dep"])
    else:
        m = _oracle(c, c["dep"], c["dep"] + q)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, SRC["amp"])
    assert r["mismatch"] == 0 and r["eta"] <= 1e-5, r
    m.step(150)
    g.step(150)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, SRC["amp"])
    assert r["mismatch"] <= 2 and r["eta"] <= 1e-4, r
    assert r["u"] <= 2e-4 and r["v"] <= 2e-4, r
    g.close()


def test_rising_source_against_oracle():
    c = _case(seed=72)
    q = cg.source_field(c["xcrd"], c["ycrd"], **SRC)
    rise = 12.5 * c["dt"]  # spread over 13 steps, the last one partial
    g = pkg.GpuGrid.from_case(c)
    g.add_source(c["xcrd"], c["ycrd"], rise_time=rise, **SRC)
    m = _oracle(c, c["dep"], c["dep"])
    ground = c["ground"]
    w_prev, el = 0.0, 0.0
    for s in range(60):
        if w_prev < 1.0:
            el += c["dt"]
            w = min(1.0, el / rise)
            H = m.cel * np.abs(m.cel) / GRAV
            wet = H > ground
            Hn = np.where(wet, H + (w - w_prev) * q, _transform(m.dep + w * q, ground))
            Hn = np.where(wet | (m.dep + w * q > ground), Hn, H)
            m.cel[...] = np.sign(Hn) * np.sqrt(GRAV * np.abs(Hn))
            w_prev = w
        m.step(1)
    g.step(60)
    cel, u, v = g.download_state()
    r = compare_state(m, cel, u, v, SRC["amp"])
    assert r["mismatch"] <= 2 and r["eta"] <= 1e-4, r
    g.close()


def test_source_arguments_are_checked():
    c = _case()
    g = pkg.GpuGrid.from_case(c)
    with pytest.raises(cg.CliffsError):
        g.add_source(c["xcrd"], c["ycrd"], **dict(SRC, ax=0.0))
    with pytest.raises(cg.CliffsError):
        g.add_source(c["xcrd"], c["ycrd"], bottom=True, rise_time=5.0, **SRC)
    g.add_source(c["xcrd"], c["ycrd"], rise_time=5.0, **SRC)
    with pytest.raises(cg.CliffsError):  # a second rising source while one is rising
        g.add_source(c["xcrd"], c["ycrd"], rise_time=5.0, **SRC)
    g.close()
