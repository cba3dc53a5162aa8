"""apply_initial_conditions.f on the device (cliffs_gpu_apply_lattice) against
the same interpolation on the oracle (oracle.apply_ic) applied on the host
before the state goes up, for every target: the surface (a deformation of
the water column, with dry cells flooding), the bottom (quake = 1), and the
velocity components; for a 2-D lattice and for lattices one node wide along
either axis, which interpolate along the other only; and a lattice two nodes
wide, which changes nothing.  After 40 steps the two runs still agree."""
import importlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
cg = pkg.cliffs_gpu
W = pkg.workloads


def _case():
    c = W.shelf_2d(seed=33, nx=300, ny=200, dx=500.0, steps=0, amp=0.0, ngauges=0)
    c["crough"] = 0.000625
    c["H0"] = c["dep"].copy()
    return c


def _lattice(c, kind):
    x, y = c["xcrd"], c["ycrd"]
    if kind == "2d":  # over the coast and part of the sea, partly outside the grid in y
        xq = np.linspace(x[100], x[-1] + 3000.0, 46)
        yq = np.linspace(y[30] - 20000.0, y[150], 51)
    elif kind == "x":
        xq, yq = np.linspace(x[150], x[-1], 40), np.array([0.0])
    elif kind == "y":
        xq, yq = np.array([0.0]), np.linspace(y[20], y[180], 33)
    else:  # two nodes wide: no change (apply_initial_conditions.f has no case for it)
        xq, yq = np.linspace(x[10], x[200], 2), np.linspace(y[10], y[150], 30)
    X, Y = np.meshgrid(xq, yq)
    q = 1.5 * np.exp(-((X - x[250]) / 15000.0) ** 2 - ((Y - y[100]) / 25000.0) ** 2) + 0.05
    return xq, yq, q


def _host_field(c, xq, yq, q):
    f = np.zeros_like(c["dep"])
    if (len(xq) > 2 and len(yq) > 2) or (len(yq) == 1 and len(xq) > 2) or (len(xq) == 1 and len(yq) > 2):
        oracle.apply_ic(xq, yq, q, c["xcrd"], c["ycrd"], f)
    return f


@pytest.mark.parametrize("kind", ["2d", "x", "y", "two"])
@pytest.mark.parametrize("target", ["surface", "bottom", "xvel", "yvel"])
def test_lattice_matches_host_interpolation(kind, target):
    c = _case()
    xq, yq, q = _lattice(c, kind)
    f = _host_field(c, xq, yq, q)
    a = pkg.GpuGrid.from_case(c)
    t = {"surface": cg.LATTICE_SURFACE, "bottom": cg.LATTICE_BOTTOM, "xvel": cg.LATTICE_XVEL,
         "yvel": cg.LATTICE_YVEL}[target]
    a.apply_lattice(c["xcrd"], c["ycrd"], xq, yq, q if target in ("surface", "bottom") else 0.1 * q, t)
    h = dict(c)
    if target == "surface":
        h["H0"] = c["dep"] + f
    elif target == "bottom":  # cliffs_main.f:193-207: cel = dep, then dep -= q
        h["H0"] = c["dep"].copy()
        h["dep"] = c["dep"] - f
    elif target == "xvel":
        h["u0"] = 0.1 * f
    else:
        h["v0"] = 0.1 * f
    b = pkg.GpuGrid.from_case(h)
    for k in range(2):
        ca, ua, va = a.download_state()
        cb, ub, vb = b.download_state()
        assert ((ca > 0.31) != (cb > 0.31)).sum() == 0, k
        assert np.abs(ca - cb).max() <= 2e-5 * max(1.0, np.abs(cb).max()), (k, np.abs(ca - cb).max())
        assert np.abs(ua - ub).max() <= 2e-5 and np.abs(va - vb).max() <= 2e-5, k
        a.step(40)
        b.step(40)
    if kind == "2d":
        assert np.abs(f).max() > 0.5  # the lattice did reach the grid
    if kind == "two":
        assert not f.any()
    a.close()
    b.close()
