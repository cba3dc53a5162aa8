"""The depth_ssl limiter on the GPU (cliffs_depth_ssl) against the oracle's
restatement of setSSLim (depth_ssl/depth_ssl.f:222-362): bit-identical
depths, the same per-passage counts and the same completion status.

Cases:
- the hand-worked lines of test_oracle_depth_ssl.py;
- random rough grids with land patches;
- a line shorter than 3 nodes;
- a rough grid at alpha = 1.5 that is still adjusting after 12 passages;
- the 2048^2 shelf bathymetry with a 50 % k^-2 perturbation.
"""
import importlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
cg = pkg.cliffs_gpu


def _check(dep, alpha=2.0, depmin=0.1):
    got = cg.depth_ssl(dep, alpha, depmin)
    ref = oracle.depth_ssl(dep, alpha, depmin)
    assert np.array_equal(got[0], ref[0])
    assert np.array_equal(got[1], ref[1])
    assert got[2] == ref[2]
    return got


@pytest.mark.parametrize("line", [[100.0, 100.0, 1.0, 100.0, 100.0], [100.0, 1.0, 1.0, 100.0],
                                  [0.05, 1.0, 100.0, 100.0], [0.05, 1.0, 0.05, 0.1, 50.0]])
def test_hand_worked_lines(line):
    a = np.array([line])
    _check(a)
    _check(a.T.copy())


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_rough_grids(seed):
    rng = np.random.default_rng(seed)
    dep = np.exp(rng.uniform(-4.0, 8.0, (97, 123)))
    dep[rng.random(dep.shape) < 0.15] = -5.0
    b, counts, _ = _check(dep)
    assert counts.sum() > 0 and not np.array_equal(b, dep)


def test_short_lines_unchanged():
    dep = np.array([[1.0, 400.0], [0.5, 900.0]])
    b, counts, st = _check(dep)
    assert np.array_equal(b, dep) and counts.sum() == 0 and st == 0


def test_incomplete_status():
    rng = np.random.default_rng(7)
    dep = np.exp(rng.uniform(-1.0, 9.0, (64, 80)))
    _check(dep, alpha=1.5)


def test_full_size_shelf():
    c = pkg.workloads.shelf_2d(seed=5, nx=2048, ny=2048, dx=100.0, steps=0, amp=0.0, ngauges=0, perturb=0.5)
    b, counts, _ = _check(c["dep"])
    assert counts[0] > 0


def _write_bathy(path, dep, dtype="f", matrix=False):
    from scipy.io import netcdf_file
    ny, nx = dep.shape
    f = netcdf_file(path, "w")
    f.history = "synthetic bathymetry"
    f.createDimension("xxx", nx)
    f.createDimension("yyy", ny)
    if matrix:
        f.createDimension("Mrow", 3)
        f.createDimension("Mclm", 3)
    vx = f.createVariable("xxx", "d", ("xxx",))
    vy = f.createVariable("yyy", "f", ("yyy",))
    vb = f.createVariable("bathy", dtype, ("yyy", "xxx"))
    vb.units = "m"
    vx[:] = np.arange(nx) * 100.0
    vy[:] = np.arange(ny) * 50.0
    vb[:] = dep
    if matrix:
        vm = f.createVariable("O2G", "d", ("Mrow", "Mclm"))
        vm[:] = np.arange(9.0).reshape(3, 3)
    f.close()


@pytest.mark.parametrize("dtype,matrix,interactive", [("f", False, False), ("d", True, False), ("f", False, True)])
def test_tool_writes_the_reference_outputs(tmp_path, dtype, matrix, interactive):
    """The depth_ssl tool on a NetCDF file: the reference's command line,
    output name, dimensions, attributes and variables; the depth as the
    oracle limits it, in the input's type."""
    import os
    import subprocess

    from scipy.io import netcdf_file
    pkg.build.build()
    tool = os.path.join(os.path.dirname(pkg.__file__), "_lib", "depth_ssl_gb300")
    rng = np.random.default_rng(11)
    dep = np.exp(rng.uniform(-3.0, 8.0, (40, 56)))
    dep[rng.random(dep.shape) < 0.1] = -10.0
    src = str(tmp_path / "area.nc")
    _write_bathy(src, dep, dtype, matrix)
    out = str(tmp_path / "out") + "/"
    os.makedirs(out)
    args = [tool, src, out, "1" if interactive else "0"]
    r = subprocess.run(args, input="3.0\n0.2\n" if interactive else "", capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "passage 1" in r.stdout
    alpha, depmin = (2.5, 0.2) if interactive else (2.0, 0.1)  # alpha clamped to 1.5-2.5
    f = netcdf_file(out + "area_ssl.nc", "r", mmap=False)
    assert f.history == b"synthetic bathymetry"
    assert f.variables["bathy"].units == b"m"
    got = f.variables["bathy"][:]
    base = dep.astype(np.float32).astype(np.float64) if dtype == "f" else dep
    ref = oracle.depth_ssl(base, alpha, depmin)[0]
    if dtype == "f":
        assert got.dtype == np.dtype(">f4") and np.array_equal(got, ref.astype(np.float32))
    else:
        assert np.array_equal(got, ref)
    assert np.array_equal(f.variables["xxx"][:], np.arange(56) * 100.0)
    if matrix:
        assert np.array_equal(f.variables["O2G"][:], np.arange(9.0).reshape(3, 3))
    f.close()
