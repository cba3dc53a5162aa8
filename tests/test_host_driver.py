"""The C++ driver (cliffs-src_gb300/host): a run read the way cliffs_main.f
reads it, and its NetCDF outputs, without a GPU (--dry-run).

The dry run reads the parameter file, grids, boundary feed and initial state
(allabout.f, MasterGrid.f, NestedGrid.f, get_boundary_feed.f,
get_initial_state.f, apply_initial_conditions.f, cliffs_main.f:131-227),
prints a JSON summary, and writes the output files (opennc4*.f) with the
initial records computed on the host.  The inputs are written by scipy's
NetCDF-3 implementation and the outputs read back by it; the expected values
come from the oracle.  The GPU run of the same driver is in
test_gpu_driver.py.
"""
import importlib
import json
import os
import subprocess
import zipfile

import numpy as np
import pytest
from scipy.io import netcdf_file

import oracle
from tests import cases

pkg = importlib.import_module("cliffs-src_gb300")
DRIVER = os.path.join(os.path.dirname(pkg.__file__), "_lib", "cliffs_gb300")
FILL = 9.9692099683868690e36


@pytest.fixture(scope="module")
def driver():
    pkg.build.build()
    assert os.path.exists(DRIVER)
    return DRIVER


def _run(driver, out, src, bprfx, aprfx, params, dry=True):
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = [driver, out, src, bprfx, aprfx, params] + (["--dry-run"] if dry else [])
    return subprocess.run(cmd, capture_output=True, text=True, timeout=600)


def _nc(path):
    return netcdf_file(path, "r", mmap=False)


def test_dry_run_reads_a_full_case(tmp_path, driver):
    d = str(tmp_path / "in") + "/"
    c = cases.write_case(d)
    ref = cases.reference_setup(c)
    out = str(tmp_path / "out" / "run")
    r = _run(driver, out, d, "bnd", "src", d + "params.txt")
    assert r.returncode == 0, r.stderr
    s = json.loads(r.stdout)
    ny, nx = c["dep"].shape
    assert (s["nx"], s["ny"], s["nests"], s["cartesian"]) == (nx, ny, 1, True)
    assert s["master"] == "master"
    assert s["steps_total"] == c["steps"] and s["seaout"] == c["seaout"] and s["ngages"] == len(c["I"])
    assert s["dt"] == c["dt"] and s["ground"] == c["ground"] and s["crough"] == c["crough"]
    # nest tables (NestedGrid.f:104-119)
    tab = oracle.NestTables(c["x"], c["y"], c["xn"], c["yn"]).as_dict()
    ch = s["children"][0]
    assert (ch["mm"], ch["nn"]) == (len(c["xn"]), len(c["yn"]))
    for k in ("W_nx", "E_nx", "S_ny", "N_ny"):
        assert ch[k] == tab[k], k
    # boundary feed start record (get_boundary_feed.f) and the source record
    assert s["bndr_input"] and s["nt"] == len(c["tinput"])
    assert s["irec"] == ref["irec"] and s["t0"] == ref["t0"]
    assert s["hinput"] and s["uinput"] and not s["vinput"]
    # initial state after apply_initial_conditions and the bottom deformation
    wet = ref["H"] > c["ground"]
    eta = ref["H"] - ref["dep"]
    assert np.isclose(s["eta_max"], eta[wet].max(), rtol=0, atol=1e-12)
    assert np.isclose(s["eta_sum"], eta[wet].sum(), rtol=1e-12)
    # the initial screenshot, subsampled (output_sea_state.f)
    ls, ts = c["lonsub"], c["latsub"]
    h = _nc(out + "_sea_h.nc")
    assert h.variables["ha"].shape == (1, (ny - 1) // ts + 1, (nx - 1) // ls + 1)
    want = np.where(wet, eta, -1e32).astype(np.float32)[::ts, ::ls]
    assert np.array_equal(h.variables["ha"][0], want)
    assert h.variables["time"][0] == ref["t0"]
    assert np.array_equal(h.variables["xxx"][:], c["x"][::ls])
    assert h.variables["ha"]._attributes["name"] == b"Surface Displacement"
    u = _nc(out + "_sea_u.nc").variables["ua"][0]
    assert np.array_equal(u, np.where(wet, ref["u"], -1e32).astype(np.float32)[::ts, ::ls])
    # gauges (output_gages.f), double precision
    g = _nc(out + "_gages.nc")
    I, J = c["I"] - 1, c["J"] - 1
    assert np.array_equal(g.variables["gage"][0], np.where(wet[J, I], eta[J, I], -1e32))
    assert np.array_equal(g.variables["u"][0], ref["u"][J, I])
    assert np.array_equal(g.variables["xxx"][:], c["x"][I])
    assert g.model == b"Cliffs"
    # max-wave file: coordinates now, fields at the first output event
    m = _nc(out + "_maxwave.nc")
    assert m.variables["MaxE"].shape == (ny, nx)
    assert np.all(m.variables["MaxE"][:] == np.float32(FILL))
    # child feed files (opennc4feed.f), no record yet
    for side, n in (("west", len(c["yn"])), ("east", len(c["yn"])), ("south", len(c["xn"])),
                    ("north", len(c["xn"]))):
        f = _nc(out + f"_child_{side}.nc")
        assert f.dimensions["pnt"] == n and f.dimensions["uvq"] == 3
        assert f.variables["vals"].shape == (0, 3, n)
    log = open(out + "_log.txt").read()
    assert "Master bathy/topo file" in log and "nested Grid 1" in log


def test_dry_run_wall_and_surface_deformation(tmp_path, driver):
    d = str(tmp_path / "in") + "/"
    c = cases.write_case(d, child=False, feed=False, quake=0, itopo=0, dwall=3.0, ngauges=0)
    ref = cases.reference_setup(c, bprfx=False)
    out = str(tmp_path / "out" / "run")
    r = _run(driver, out, d, "0", "src", d + "params.txt")
    assert r.returncode == 0, r.stderr
    s = json.loads(r.stdout)
    assert not s["bndr_input"] and s["irec"] == 1 and s["t0"] == c["tsrc"][0]
    assert s["dep_min"] == -999.0  # the wall at dwall (cliffs_main.f:131-137)
    wet = ref["H"] > c["ground"]
    eta = ref["H"] - ref["dep"]
    assert np.isclose(s["eta_sum"], eta[wet].sum(), rtol=1e-12)
    h = _nc(out + "_sea_h.nc").variables["ha"][0]
    assert np.array_equal(h, np.where(wet, eta, -1e32).astype(np.float32)[::3, ::2])
    assert not os.path.exists(out + "_gages.nc")


@pytest.mark.parametrize("what", ["no_input", "missing_grid", "gage_outside", "below_threshold", "short_params"])
def test_driver_errors(tmp_path, driver, what):
    d = str(tmp_path / "in") + "/"
    cases.write_case(d, child=False)
    p = d + "params.txt"
    lines = open(p).read().splitlines()
    bprfx, aprfx = "bnd", "src"
    if what == "no_input":
        bprfx = aprfx = "0"
        msg = "no input of any kind"
    elif what == "missing_grid":
        os.remove(d + "master.nc")
        msg = "cannot open"
    elif what == "gage_outside":
        lines[-1] = "9999 1"
        msg = "outside the grid"
    elif what == "below_threshold":
        lines[3] = "100.0\tStill sea threshold on the boundary (m)"
        msg = "bndr signal below threshold"
    else:
        lines = lines[:8]
        msg = "parameter file ends early"
    open(p, "w").write("\n".join(lines) + "\n")
    out = str(tmp_path / "out" / "run")
    r = _run(driver, out, d, bprfx, aprfx, p)
    assert r.returncode == 1
    assert msg in r.stderr, r.stderr
    assert msg in open(out + "_log.txt").read()


def test_help_without_arguments(driver):
    r = subprocess.run([driver], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "Help" in r.stdout


def test_reference_example_slpbeach(tmp_path, driver, reference_dir):
    """The reference's own 1-D example (Examples/slpbeach.zip), read from the
    archive: grid, parameter file and the solitary-wave source."""
    z = os.path.join(reference_dir, "Examples", "slpbeach.zip")
    if not os.path.exists(z):
        pytest.skip("reference examples not present")
    zipfile.ZipFile(z).extractall(tmp_path)
    d = str(tmp_path / "slpbeach") + "/"
    out = str(tmp_path / "out" / "slp")
    r = _run(driver, out, d, "0", "solitary.0185", d + "slpbeach_params.txt")
    assert r.returncode == 0, r.stderr
    s = json.loads(r.stdout)
    grid = _nc(d + "slpbeach1D.nc")
    names = list(grid.variables)
    x = grid.variables[names[0]][:].astype(np.float64)
    y = grid.variables[names[1]][:].astype(np.float64)
    dep = grid.variables[names[2]][:].astype(np.float64).reshape(len(y), len(x))
    assert (s["nx"], s["ny"]) == (len(x), len(y))
    vals = [ln.split()[0] for ln in open(d + "slpbeach_params.txt").read().splitlines() if ln.strip()]
    assert s["ground"] == float(vals[4]) and s["dt"] == float(vals[8]) and s["steps_total"] == int(vals[9])
    src = _nc(d + "solitary.0185_h.nc")
    sv = list(src.variables)
    xs, ys = src.variables["xxx"][:], src.variables["yyy"][:]
    q = src.variables[sv[-1]][0].astype(np.float32).astype(np.float64)
    H = dep.copy()
    oracle.apply_ic(xs, ys, q, x, y, H)
    wet = H > s["ground"]
    h = _nc(out + "_sea_h.nc").variables["ha"][0]
    assert np.array_equal(h, np.where(wet, H - dep, -1e32).astype(np.float32))
    assert 0.015 < s["eta_max"] < 0.02  # the example's H/d = 0.0185 wave on a 1 m shelf
