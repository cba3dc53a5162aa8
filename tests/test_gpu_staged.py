"""The staged sweep kernels (persistent, windows brought into shared memory by
bulk copies one tile ahead) against the tiled ones (one block per tile,
loads into registers): bit-identical states and max-wave fields over runs that
reach every path, and the failure-detection check of the stage waits.

Cases: a shelf whose wave runs up the coast (the general path of both
sweeps), a spherical grid whose sizes are multiples of neither the x tile
(512 cells) nor the y tile (32 x 16), a 1-D channel (x-sweep alone, max-wave
fused into it) and a grid 3 cells wide.
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
    a.set_sweep_kernel(cg.STAGED)
    b = pkg.GpuGrid.from_case(case)
    b.set_sweep_kernel(cg.TILED)  # the default
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


@pytest.mark.parametrize("make,steps", [(_shelf, 300), (_sphere, 120), (_narrow, 200)])
def test_staged_equals_tiled(make, steps):
    a, b = _pair(make())
    for n in (1, steps - 1):
        a.step(n)
        b.step(n)
        _same(a, b)
    a.close()
    b.close()


def test_staged_equals_tiled_channel():
    c = W.channel_1d(seed=3, n=2000, steps=0)
    a, b = _pair(c)
    a.step(1500)
    b.step(1500)
    _same(a, b)
    me, _ = a.maxwave()
    assert me.max() > 0.01  # the max-wave update ran in the x-sweep
    a.close()
    b.close()


def test_stage_wait_timeout_reported():
    """The copy waits of one staged x-sweep and of one tiled y-sweep expect
    bytes no copy brings: every wait runs out after 50 ms, the host reads
    CLIFFS_ERR_TIMEOUT (both sweeps reported it), the state is unchanged and
    the next steps run as usual."""
    a, b = _pair(_shelf())
    a.step(20)
    b.step(20)
    before = a.download_state()
    assert a.check_stage_timeout(50) == -7
    after = a.download_state()
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    assert a.status()[0] == 0  # the check cleared its own flag
    a.step(30)
    b.step(30)
    _same(a, b)
    a.close()
    b.close()
