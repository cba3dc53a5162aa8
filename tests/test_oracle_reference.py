"""The oracle's line update against the reference's own code.

oracle/ref_f2c.py translates the reference's subroutine cliffs
(cliffs.f:17-346) from the checkout's source into C and compiles it
(oracle/_ref).  Here the oracle's restatement (oracle/cliffs_oracle.c,
orc_line) and that translation advance the same lines from the same state,
and every value of cel, xvel and yvel must agree bit for bit:

- random lines on a small grid, both directions, with sea and land nodes,
  dry cells, flooding fronts on either side, supercritical flow, open and
  forced line ends, non-uniform spacing and the spherical metric term;
- every row and every column of a shelf basin at several times of a run
  from a Gaussian source (the wet/dry fronts the time loop produces).

Runs where the reference checkout is present (the build container); the
GPU hosts have none.
"""
import ctypes

import numpy as np
import pytest

import oracle
from tests.conftest import REFERENCE

_dp = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def ref(reference_dir):
    from oracle.ref_f2c import build

    L = ctypes.CDLL(build(reference_dir))
    f = L.ref_cliffs
    f.restype = None
    f.argtypes = [ctypes.c_int] * 6 + [_dp] * 9 + [ctypes.c_double] * 5
    return f


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _compare_line(ref, m, iu, irw):
    """One line through both; returns the number of differing values."""
    cel, xv, yv = m.cel.copy(), m.xvel.copy(), m.yvel.copy()
    ref(iu, irw, m.nx if iu == 1 else m.ny, m.nx, m.ny, m.mx, _p(m.dep), _p(cel), _p(xv), _p(yv),
        _p(m.s1), _p(m.s2), _p(m.zeta), _p(m.edge1), _p(m.edge2), oracle.GRAV, m.g.ground, m.g.crough, m.g.dt,
        m.celmin)
    m.line(iu, irw)
    assert not m.seg_overflow
    return int((cel.view(np.int64) != m.cel.view(np.int64)).sum() + (xv.view(np.int64) != m.xvel.view(np.int64)).sum()
               + (yv.view(np.int64) != m.yvel.view(np.int64)).sum())


def _random_grid(rng, nx, ny, spherical):
    # sea and land nodes in runs, so that lines hold shorelines and dry patches
    dep = np.empty((ny, nx))
    for j in range(ny):
        sign = np.where(rng.random(nx) < 0.25, -1.0, 1.0)
        sign = np.where(np.convolve(sign, np.ones(3) / 3, "same") < 0, -1.0, 1.0)
        dep[j] = sign * rng.uniform(0.05, 3.0, nx)
    ground = 0.01
    # total depth: sea nodes wet, land nodes dry or wet by a thin layer
    H = np.where(dep > 0, dep + rng.normal(0, 0.1, dep.shape), 0.0)
    wet_land = (dep < 0) & (rng.random(dep.shape) < 0.3)
    H = np.where(wet_land, rng.uniform(0.0, 0.1, dep.shape), H)
    H = np.where(rng.random(dep.shape) < 0.05, rng.uniform(0.0, 0.02, dep.shape), H)  # near the threshold
    H = np.maximum(H, 0.0)
    u = rng.normal(0, 0.3, dep.shape)
    v = rng.normal(0, 0.3, dep.shape)
    fast = rng.random(dep.shape) < 0.03  # supercritical spots
    u = np.where(fast, rng.choice([-1, 1], dep.shape) * rng.uniform(2, 6, dep.shape), u)
    s1 = rng.uniform(0.8, 1.2, (ny, nx - 1))
    s2 = rng.uniform(0.8, 1.2, ny - 1)
    zeta = rng.normal(0, 1e-3, ny) if spherical else np.zeros(ny)
    m = oracle.Model(dep, s1, s2, zeta, ground=ground, crough=0.0025, dt=0.05, cel=H, xvel=u, yvel=v)
    # forced or open line ends: elevation, normal and tangential velocity
    for e in (m.edge1, m.edge2):
        e[0] = rng.normal(0, 0.2, m.mx)
        e[1] = rng.normal(0, 0.2, m.mx)
        e[2] = np.where(rng.random(m.mx) < 0.5, rng.normal(0, 0.1, m.mx), 0.0)
    return m


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("spherical", [False, True])
def test_random_lines_bit_identical(ref, seed, spherical):
    rng = np.random.default_rng(1000 + seed)
    m = _random_grid(rng, 57, 23, spherical)
    bad = changed = mixed = 0
    for iu, nl in ((1, m.ny), (2, m.nx)):
        for irw in range(1, nl + 1):
            line = m.cel[irw - 1] if iu == 1 else m.cel[:, irw - 1]
            mixed += int((line <= m.celmin).any() and (line > m.celmin).any())
            before = m.cel.copy()
            bad += _compare_line(ref, m, iu, irw)
            changed += int((before != m.cel).any())
    assert bad == 0
    # the lines hold wet/dry fronts and the update moved them
    assert mixed >= (m.nx + m.ny) // 2 and changed >= (m.nx + m.ny) // 2, (mixed, changed)


def test_shelf_run_lines_bit_identical(ref):
    import importlib

    W = importlib.import_module("cliffs-src_gb300.workloads")
    case = W.shelf_2d(seed=2, nx=96, ny=80, dx=100.0, steps=400, ngauges=4)
    case["crough"] = 0.000625
    s1, s2, zeta = oracle.metrics(case["xcrd"], case["ycrd"], True)
    m = oracle.Model(case["dep"], s1, s2, zeta, ground=case["ground"], crough=case["crough"], dt=case["dt"],
                     cel=case["H0"])
    checked = 0
    for target in (0, 60, 150, 300):
        m.step(target - m.istep)
        snap = (m.cel.copy(), m.xvel.copy(), m.yvel.copy())
        for iu, nl in ((1, m.ny), (2, m.nx)):
            for irw in range(1, nl + 1):
                assert _compare_line(ref, m, iu, irw) == 0, (target, iu, irw)
                checked += 1
                m.cel[...], m.xvel[...], m.yvel[...] = snap  # every line from the same state
    assert checked == 4 * (96 + 80)
    # the run reached land: some line went through the wet/dry scan with a front
    assert (m.cel <= m.celmin).any() and (m.cel > m.celmin).any()
