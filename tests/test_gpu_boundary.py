"""ComputeBoundaryInput on the GPU (cliffs_boundary_scan, cliffs_boundary_edges
and the cmpboundary_gb300 tool) against the oracle's restatement of
cmpboundary/scan4wave.f, get_sea_state.f and InterpolateOntoBndr.f:
bit-identical records, the reference's quirks (a first signal at the last
record counts as none, centimetres scaled in single precision, missing values
as 0), and the tool's command line, file names and NetCDF layout."""
import importlib
import os
import subprocess

import numpy as np
import pytest

import oracle

pkg = importlib.import_module("cliffs-src_gb300")
G = pkg.cliffs_gpu

pytestmark = pytest.mark.gpu


def _footprint(t, field):
    d = t.as_dict()
    return np.ascontiguousarray(field[:, d["S_ny"] - 1:d["N_ny"] + 1, d["W_nx"] - 1:d["E_nx"] + 1])


@pytest.mark.parametrize("seed,shape", [(0, (1, 2, 2)), (1, (9, 17, 33)), (2, (300, 61, 47)), (3, (40, 700, 900))])
def test_scan_matches_oracle(seed, shape):
    rng = np.random.default_rng(seed)
    nt = shape[0]
    c = rng.normal(0.0, 1e-3, shape).astype(np.float32)
    c[rng.random(shape) < 0.1] = -1.0e25
    for k in range(nt):                       # the signal grows record by record
        c[k] *= 1.0 + 10.0 * k
    for cuke in (0.0, 1e-3, 0.02, 0.3, 10.0):
        assert G.boundary_scan(c, cuke) == oracle.boundary_scan(c, cuke)


def test_scan_quirks():
    c = np.zeros((7, 3, 4), np.float32)
    assert G.boundary_scan(c, 0.01) == 8      # none: nt + 1
    c[6, 2, 3] = -1.0
    assert G.boundary_scan(c, 0.01) == 7      # at the last record: nt, also 'no signal'
    c[2, 0, 0] = 0.5
    assert G.boundary_scan(c, 0.5) == 7       # equal to cuke is still sea
    c[1, 1, 1] = -1.0e10                      # -1e10 is a value; below it is missing
    c[0, 1, 1] = -1.0e11
    assert G.boundary_scan(c, 0.5) == 2


def _case(seed, n=(61, 46), m=(211, 187), nt=9):
    rng = np.random.default_rng(seed)
    x = np.cumsum(rng.uniform(0.2, 0.4, n[0])) + 130.0
    y = np.cumsum(rng.uniform(0.2, 0.4, n[1])) + 30.0
    xn = np.linspace(rng.uniform(x[1], x[5]), rng.uniform(x[-6], x[-1]), m[0])
    yn = np.linspace(rng.uniform(y[0], y[4]), rng.uniform(y[-5], y[-1]), m[1])
    t = oracle.NestTables(x, y, xn, yn)
    field = rng.normal(0.0, 50.0, (3, nt, n[1], n[0])).astype(np.float32)
    field[rng.random(field.shape) < 0.05] = -1.0e30
    return t, [_footprint(t, f) for f in field]


@pytest.mark.parametrize("seed,scale", [(0, 1.0), (1, 0.01), (2, 1.0)])
def test_edges_match_oracle(seed, scale):
    t, cubes = _case(seed)
    got = G.boundary_edges(t.as_dict(), cubes, scale)
    ref = oracle.boundary_edges(t, cubes, scale)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


def test_edges_large_footprint():
    """A 1/60 degree target over a 1/12 degree lattice, 64 records."""
    x = np.arange(0.0, 40.0, 1 / 12)
    y = np.arange(-10.0, 20.0, 1 / 12)
    xn = np.arange(5.0, 30.0, 1 / 60)
    yn = np.arange(-2.0, 15.0, 1 / 60)
    t = oracle.NestTables(x, y, xn, yn)
    rng = np.random.default_rng(5)
    cubes = [_footprint(t, rng.normal(0, 1, (64, len(y), len(x))).astype(np.float32)) for _ in range(3)]
    got = G.boundary_edges(t.as_dict(), cubes, 0.01)
    ref = oracle.boundary_edges(t, cubes, 0.01)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


def test_edges_refuse_rows_outside_the_cube():
    t, cubes = _case(4)
    small = [np.ascontiguousarray(c[:, :-1, :]) for c in cubes]   # north row cut off
    with pytest.raises(G.CliffsError):
        G.boundary_edges(t.as_dict(), small, 1.0)


# ---- the tool ---------------------------------------------------------------

def _write_sea(path, x, y, t, field):
    from scipy.io import netcdf_file
    f = netcdf_file(path, "w")
    f.createDimension("time", None)
    f.createDimension("lat", len(y))
    f.createDimension("lon", len(x))
    vt = f.createVariable("time", "d", ("time",))
    vy = f.createVariable("lat", "d", ("lat",))
    vx = f.createVariable("lon", "d", ("lon",))
    vf = f.createVariable("field", "f", ("time", "lat", "lon"))
    vy[:] = y
    vx[:] = x
    vt[:] = t
    vf[:] = field
    f.close()


def _write_grid(path, xn, yn):
    from scipy.io import netcdf_file
    f = netcdf_file(path, "w")
    f.createDimension("xxx", len(xn))
    f.createDimension("yyy", len(yn))
    f.createVariable("xxx", "d", ("xxx",))[:] = xn
    f.createVariable("yyy", "f", ("yyy",))[:] = yn
    f.createVariable("z", "f", ("yyy", "xxx"))[:] = np.ones((len(yn), len(xn)))
    f.close()


def _tool():
    pkg.build.build()
    return os.path.join(os.path.dirname(pkg.__file__), "_lib", "cmpboundary_gb300")


def _setup(tmp_path, first_signal, nt=12):
    rng = np.random.default_rng(21)
    x = np.linspace(140.0, 146.0, 73)
    y = np.linspace(35.0, 40.0, 61)
    tsec = np.arange(nt) * 60.0
    fields = {}
    for c in "huv":
        f = rng.normal(0.0, 1e-4, (nt, len(y), len(x))).astype(np.float32)
        f[rng.random(f.shape) < 0.02] = -1.0e20
        if first_signal <= nt:
            f[first_signal - 1:] += rng.normal(0.0, 2.0, f[first_signal - 1:].shape).astype(np.float32)
        fields[c] = f
        _write_sea(str(tmp_path / f"run_{c}.nc"), x, y, tsec, f)
    xn = np.linspace(141.3, 143.9, 95)
    yn = (np.linspace(36.2, 38.7, 76)).astype(np.float32).astype(np.float64)
    _write_grid(str(tmp_path / "target.nc"), xn, yn)
    return x, y, tsec, xn, yn, fields


def _run(tmp_path, units, cuke=0.05, name="run_h.nc"):
    out = str(tmp_path / "out")
    os.makedirs(out, exist_ok=True)
    args = [_tool(), str(tmp_path / name), str(tmp_path / "target.nc"), out + "/case", units]
    return subprocess.run(args, input=f"{cuke}\n", capture_output=True, text=True, timeout=300), out + "/case_target"


@pytest.mark.parametrize("units,first", [("m", 5), ("cm", 1), ("m", 12)])
def test_tool_writes_the_reference_outputs(tmp_path, units, first):
    from scipy.io import netcdf_file
    x, y, tsec, xn, yn, fields = _setup(tmp_path, first)
    r, base = _run(tmp_path, units)
    assert r.returncode == 0, r.stderr
    nt = len(tsec)
    t = oracle.NestTables(x, y, xn, yn)
    it = oracle.boundary_scan(_footprint(t, fields["h"]), 0.05)
    assert it == first
    assert ("no signal above treshold" in r.stdout) == (it >= nt)
    cubes = [_footprint(t, fields[c])[it - 1:] for c in "uvh"]
    ref = oracle.boundary_edges(t, cubes, 1.0 if units == "m" else 0.01)
    for edge, want, npnt in zip(("west", "east", "south", "north"), ref, (len(yn), len(yn), len(xn), len(xn))):
        f = netcdf_file(f"{base}_{edge}.nc", "r", mmap=False)
        assert f.dimensions["pnt"] == npnt and f.dimensions["uvq"] == 3
        assert f.variables["vals"].dimensions == ("tim", "uvq", "pnt")
        assert np.array_equal(f.variables["time"][:], tsec[it - 1:])
        assert np.array_equal(f.variables["vals"][:], want), edge
        f.close()


def test_tool_without_signal_writes_no_records(tmp_path):
    from scipy.io import netcdf_file
    _setup(tmp_path, first_signal=99)
    r, base = _run(tmp_path, "m", cuke=1.0)
    assert r.returncode == 0, r.stderr
    assert "no signal above treshold" in r.stdout
    f = netcdf_file(f"{base}_north.nc", "r", mmap=False)
    assert f.variables["vals"].shape == (0, 3, 95) and f.variables["time"].shape == (0,)
    f.close()


def test_tool_refusals(tmp_path):
    _setup(tmp_path, first_signal=3)
    # the 'h' of the name may be neither its first nor its last character
    os.rename(str(tmp_path / "run_h.nc"), str(tmp_path / "h_run.nc"))
    r, _ = _run(tmp_path, "m", name="h_run.nc")
    assert r.returncode == 1 and "Wrong naming for input dataset" in r.stdout
    os.rename(str(tmp_path / "h_run.nc"), str(tmp_path / "run_h.nc"))
    # the target must lie within the source lattice
    _write_grid(str(tmp_path / "target.nc"), np.linspace(139.0, 143.0, 20), np.linspace(36.0, 38.0, 20))
    r, _ = _run(tmp_path, "m")
    assert r.returncode == 1 and "not within source grid limits" in r.stdout
    # help
    r = subprocess.run([_tool()], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Help:" in r.stdout


def test_pipeline_parent_screenshots_force_a_child(tmp_path):
    """The reference's workflow for an externally forced grid, all of it on
    the GPU: a coarse run writes its screenshots (cliffs_gb300), the edge
    records of a finer target grid are built from them (cmpboundary_gb300,
    bit-identical to the oracle on the files as written), and the target grid
    runs forced by those files."""
    from scipy.interpolate import RegularGridInterpolator
    from scipy.io import netcdf_file

    from tests import cases
    driver = os.path.join(os.path.dirname(pkg.__file__), "_lib", "cliffs_gb300")
    d = str(tmp_path / "parent") + "/"
    c = cases.write_case(d, steps=240, seaout=20, gout=20, maxout=120, bndout=20, child=False, feed=False)
    pout = str(tmp_path / "pout" / "run")
    os.makedirs(os.path.dirname(pout))
    r = subprocess.run([driver, pout, d, "0", "src", d + "params.txt"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    # the target: a 1/3 refinement of part of the parent, its bathymetry interpolated
    x, y, dx = c["x"], c["y"], c["x"][1] - c["x"][0]
    xn = np.arange(x[60] + 150.0, x[130], dx / 3)
    yn = np.arange(y[40] + 90.0, y[110], dx / 3)
    interp = RegularGridInterpolator((y, x), c["dep"])
    Y, X = np.meshgrid(yn, xn, indexing="ij")
    depn = interp(np.stack([Y.ravel(), X.ravel()], 1)).reshape(Y.shape).astype(np.float32)
    cd = str(tmp_path / "child") + "/"
    os.makedirs(cd)
    cases._nc_grid(cd + "tgt.nc", xn, yn, depn)
    r = subprocess.run([_tool(), pout + "_sea_h.nc", cd + "tgt.nc", cd + "bnd", "m"], input="0.001\n",
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    # the edge records against the oracle, from the screenshots as written
    fields = {}
    for k in "huv":
        f = netcdf_file(f"{pout}_sea_{k}.nc", "r", mmap=False)
        xs, ys, ts = f.variables["xxx"][:].copy(), f.variables["yyy"][:].copy(), f.variables["time"][:].copy()
        fields[k] = f.variables[k + "a"][:].astype(np.float32)
        f.close()
    t = oracle.NestTables(xs, ys, xn, yn)
    it = oracle.boundary_scan(_footprint(t, fields["h"]), 0.001)
    assert 1 <= it < len(ts)
    ref = oracle.boundary_edges(t, [_footprint(t, fields[k])[it - 1:] for k in "uvh"], 1.0)
    for edge, want in zip(("west", "east", "south", "north"), ref):
        f = netcdf_file(f"{cd}bnd_tgt_{edge}.nc", "r", mmap=False)
        assert np.array_equal(f.variables["vals"][:], want), edge
        assert np.array_equal(f.variables["time"][:], ts[it - 1:])
        f.close()
    # the target grid, forced by those files
    new = {"time step (sec)": f"{c['dt'] / 3!r}", "total amount of steps": "300", "1 - to deform bottom": "0",
           "N gages": "0"}
    lines = []
    for s in open(d + "params.txt").read().splitlines():
        key = s.split("\t", 1)[-1]
        lines.append(new[key] + "\t" + key if key in new else "tgt.nc" if s == "master.nc" else s)
        if key == "N gages":
            break
    with open(cd + "params.txt", "w") as f:
        f.write("\n".join(lines) + "\n")
    cout = str(tmp_path / "cout" / "run")
    os.makedirs(os.path.dirname(cout))
    r = subprocess.run([driver, cout, cd, "bnd", "0", cd + "params.txt"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr + open(cout + "_log.txt").read()
    f = netcdf_file(cout + "_maxwave.nc", "r", mmap=False)
    me = f.variables["MaxE"][:]
    f.close()
    wet = me > -1e30
    assert wet.mean() > 0.5 and np.isfinite(me[wet]).all() and np.abs(me[wet]).max() < 20.0
