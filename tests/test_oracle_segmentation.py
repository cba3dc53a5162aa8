"""The per-cell wet/dry rules equal the reference's serial segment scan.

The GPU kernels decide segments, flooding, shoreline ghosts and the angle
limiter from each cell's neighbours (cells i-1..i+1) instead of the serial
left-to-right scan of cliffs.f:65-111.  orc_line_local applies those rules
with the reference's own FP64 arithmetic, so on every line it must produce
bit-identical cel/xvel/yvel to orc_line, the verbatim scan.
"""
import itertools

import numpy as np
import pytest

import oracle
from tests.lines import random_grid, random_spacing


def _model(dep, cel, u, v, dx, ground, crough=0.0, zeta=None, dt=0.05):
    ny, nx = dep.shape
    s1 = np.tile(dx, (ny, 1)) if nx > 2 else None
    s2 = np.ones(ny - 1) if ny > 2 else None
    z = zeta if zeta is not None else (np.zeros(ny) if ny > 2 else None)
    m = oracle.Model(dep, s1, s2, z, ground=ground, crough=crough, dt=dt)
    # install celerity directly (the constructor transformed H)
    m.cel[...] = cel
    m.xvel[...] = u
    m.yvel[...] = v
    return m


def _equal(a, b):
    return np.array_equal(a.cel, b.cel) and np.array_equal(a.xvel, b.xvel) and \
        np.array_equal(a.yvel, b.yvel)


@pytest.mark.parametrize("seed", range(6))
def test_local_rules_match_scan_random(seed):
    rng = np.random.default_rng(1000 + seed)
    ground = [0.01, 0.003, 0.1][seed % 3]
    for n in (3, 4, 5, 7, 12, 33, 80):
        dep, cel, u, v = random_grid(rng, 300, n, ground=ground)
        dx = random_spacing(rng, n)
        a = _model(dep, cel, u, v, dx, ground, crough=0.002 * (seed % 2))
        b = _model(dep, cel, u, v, dx, ground, crough=0.002 * (seed % 2))
        # forced edges: eta, u, v of the feed for every row
        e1 = rng.uniform(-0.3, 0.3, (3, a.mx))
        e2 = rng.uniform(-0.3, 0.3, (3, a.mx))
        for m in (a, b):
            m.edge1[...] = e1
            m.edge2[...] = e2
        a.sweep(1, local=False)
        b.sweep(1, local=True)
        assert _equal(a, b), f"x-sweep mismatch n={n} seed={seed}"
        assert not a.seg_overflow


@pytest.mark.parametrize("seed", range(3))
def test_local_rules_match_scan_ysweep(seed):
    rng = np.random.default_rng(2000 + seed)
    ground = 0.01
    for n in (3, 6, 17, 64):
        # build a grid whose columns are random lines: transpose the row generator
        dep, cel, u, v = random_grid(rng, 40, n, ground=ground)
        dep, cel, u, v = (np.ascontiguousarray(x.T) for x in (dep, cel, u, v))
        ny, nx = dep.shape
        zeta = rng.uniform(-2e-8, 2e-8, ny)
        dx = np.ones(nx - 1)
        a = _model(dep, cel, u, v, dx, ground, zeta=zeta)
        b = _model(dep, cel, u, v, dx, ground, zeta=zeta)
        s2 = random_spacing(rng, ny)
        a.s2[...] = s2
        b.s2[...] = s2
        a.sweep(2, local=False)
        b.sweep(2, local=True)
        assert _equal(a, b), f"y-sweep mismatch n={n} seed={seed}"


def test_local_rules_match_scan_exhaustive_small():
    """Every land/water and flow-direction pattern on lines of 3..6 cells."""
    ground = 0.01
    celmin = np.sqrt(oracle.GRAV * ground)
    rng = np.random.default_rng(7)
    for n in range(3, 7):
        pats = list(itertools.product([0, 1, 2], repeat=n))  # 0 dry, 1 shallow wet, 2 deep wet
        upat = list(itertools.product([-1.0, 1.0], repeat=n))
        rows = []
        for p in pats:
            for uu in rng.choice(len(upat), 4, replace=False):
                rows.append((p, upat[uu]))
        L = len(rows)
        dep = np.zeros((L + 2, n))
        cel = np.zeros((L + 2, n))
        u = np.zeros((L + 2, n))
        for r, (p, uu) in enumerate(rows, start=1):
            p = np.array(p)
            dep[r] = np.where(p == 0, -0.02, np.where(p == 1, 0.004, 0.5))
            H = np.where(p == 0, 0.0, np.where(p == 1, 0.05, 0.55))
            cel[r] = np.where(p == 0, 0.0, np.sqrt(oracle.GRAV * H))
            u[r] = np.array(uu) * np.where(p == 2, 0.3, 0.8)
        v = np.ones_like(u) * 0.1
        dep = dep.astype(np.float32).astype(np.float64)
        dx = np.ones(n - 1)
        a = _model(dep, cel, u, v, dx, ground)
        b = _model(dep, cel, u, v, dx, ground)
        a.sweep(1, local=False)
        b.sweep(1, local=True)
        assert _equal(a, b), f"exhaustive mismatch n={n}"
        assert celmin > 0


def test_fully_dry_line_untouched():
    """cliffs.f:113: a line without a wet cell is not modified at all."""
    ground = 0.01
    celmin = np.sqrt(oracle.GRAV * ground)
    n = 10
    dep = np.full((3, n), -1.0)
    cel = np.full((3, n), 0.5 * celmin)
    u = np.full((3, n), 0.7)
    v = np.full((3, n), -0.2)
    for local in (False, True):
        m = _model(dep, cel, u, v, np.ones(n - 1), ground)
        m.sweep(1, local=local)
        assert np.array_equal(m.cel[1], cel[1])
        assert np.array_equal(m.xvel[1], u[1])
    # one wet cell anywhere zeroes every dry cell of the line
    cel2 = cel.copy()
    cel2[1, 7] = 2.0
    dep2 = dep.copy()
    dep2[1, 6:9] = 0.3
    m = _model(dep2, cel2, u, v, np.ones(n - 1), ground)
    m.sweep(1)
    assert m.cel[1, 0] == 0.0 and m.xvel[1, 0] == 0.0 and m.yvel[1, 0] == 0.0
