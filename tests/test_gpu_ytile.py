"""The y-sweep with its tiles staged in shared memory by tensor-map copies
(tile_y_kernel, the default tiled kernels) against the y-sweep that loads its
window straight into registers (CLIFFS_SWEEP_DIRECT): bit-identical states
and max-wave fields.

Cases: a shelf whose wave runs up the coast (listed cells finished into the
tile), a spherical grid with the metric term whose sizes are multiples of
neither 32 columns nor 16 rows (tiles clipped at the grid's edges, rows
outside the grid read 0), a grid 3 cells wide, a grid 9 rows high (one band,
most of it outside the grid), a grid forced at all four edges (edge tables
read by the tile), and the 2048 x 2048 benchmark shelf.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads
cg = pkg.cliffs_gpu


def _pair(case):
    a = pkg.GpuGrid.from_case(case)
    a.set_sweep_kernel(cg.TILED)  # the default
    b = pkg.GpuGrid.from_case(case)
    b.set_sweep_kernel(cg.DIRECT)
    return a, b


def _same(a, b):
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)
    assert a.status()[0] == 0 and b.status()[0] == 0


def _shelf():
    c = W.shelf_2d(seed=81, nx=300, ny=220, dx=500.0, steps=0, ngauges=0, axes_km=(30, 15),
                   centre_km=(120.0, 55.0))
    c["crough"] = 0.000625
    return c


def _sphere():
    c = W.sphere_2d(seed=5, nx=1100, ny=70, lat=(-30.0, 40.0), dlon=1.0 / 30.0, steps=0, ngauges=0,
                    axes_nodes=(80, 30))
    c["crough"] = 0.000625
    return c


def _narrow():
    """3 x 500 channel along y: 50 m deep, a beach rising to 2 m of land over
    the last 60 rows, a Gaussian hump of 1 m."""
    ny, dx = 500, 200.0
    y = np.arange(ny) * dx
    d = np.where(np.arange(ny) < ny - 60, 50.0, 50.0 - 52.0 * (np.arange(ny) - (ny - 60)) / 59.0)
    dep = np.repeat(W._f32(d)[:, None], 3, axis=1)
    H0 = dep + np.exp(-((y - 0.75 * ny * dx) / 5000.0) ** 2)[:, None]
    return dict(xcrd=np.arange(3) * dx, ycrd=y, cartesian=True, dep=dep, H0=H0, u0=np.zeros_like(dep),
                v0=np.zeros_like(dep), ground=0.01, crough=0.0, dt=float(0.8 * dx / np.sqrt(9.8 * 50.0)))


def _short():
    """9 rows, 70 columns: one band of 16 rows, partly outside the grid."""
    c = W.shelf_2d(seed=12, nx=70, ny=9, dx=2000.0, steps=0, ngauges=0, axes_km=(40, 6), centre_km=(60.0, 9.0))
    c["crough"] = 0.000625
    return c


@pytest.mark.parametrize("make,steps", [(_shelf, 300), (_sphere, 120), (_narrow, 200), (_short, 150)])
def test_tiled_y_equals_direct(make, steps):
    a, b = _pair(make())
    for n in (1, steps - 1):
        a.step(n)
        b.step(n)
        _same(a, b)
    a.close()
    b.close()


def _records(nt, n, tin, amp, phase):
    t = tin[:, None]
    s = np.linspace(0.0, 1.0, n)[None, :]
    eta = amp * np.sin(2 * np.pi * (t / (tin[-1] + 1.0) + s + phase))
    rec = np.zeros((nt, 3, n))
    rec[:, 0] = 0.3 * eta
    rec[:, 1] = 0.1 * eta
    rec[:, 2] = eta
    return rec


def test_tiled_y_equals_direct_forced():
    case = W.shelf_2d(seed=21, nx=160, ny=120, dx=1000.0, steps=0, amp=0.0, ngauges=0, perturb=0.02)
    ny, nx = case["dep"].shape
    nt = 30
    tin = np.arange(nt) * 8 * case["dt"]
    feed = (_records(nt, ny, tin, 0.4, 0.0), _records(nt, ny, tin, 0.1, 0.3), _records(nt, nx, tin, 0.2, 0.1),
            _records(nt, nx, tin, 0.05, 0.6))
    a, b = _pair(case)
    for g in (a, b):
        g.set_feed(tin, *feed, irec=2, freeze=True)
        g.t.value = tin[1]
    ra, rb = a.step(150), b.step(150)
    assert ra == rb
    _same(a, b)
    a.close()
    b.close()


def test_tiled_y_equals_direct_2048():
    c = W.shelf_2d(seed=0, nx=2048, ny=2048, dx=100.0, steps=3000, ngauges=0)
    c["crough"] = 0.000625
    a, b = _pair(c)
    a.step(200)
    b.step(200)
    _same(a, b)
    a.close()
    b.close()
