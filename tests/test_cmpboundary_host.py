"""Host side of the cmpboundary_gb300 tool (ComputeBoundaryInput,
cmpboundary/cmpboundary.f:44-190), on the CPU: the help line, the still-sea
threshold read from standard input, the lattices read from NetCDF, the
refusal of a target outside the source lattice, and a loud failure where the
device part would run but no GPU is present (no CPU fallback)."""
import os
import subprocess

import numpy as np
import pytest

from test_gpu_boundary import _run, _setup, _tool, _write_grid


def test_help():
    r = subprocess.run([_tool()], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Help:" in r.stdout and "<units(m/cm)>" in r.stdout


def test_target_outside_the_lattice(tmp_path):
    _setup(tmp_path, first_signal=3)
    _write_grid(str(tmp_path / "target.nc"), np.linspace(141.0, 143.0, 20), np.linspace(36.0, 40.5, 20))
    r, base = _run(tmp_path, "m")
    assert r.returncode == 1
    assert "Nodes in Sea State Dataset (lon/lat/time): 73 61 12" in r.stdout
    assert "Target area lon/lat limits: 141 143 36 40.5" in r.stdout
    assert "not within source grid limits" in r.stdout
    assert not os.path.exists(base + "_west.nc")


def test_no_threshold_on_stdin(tmp_path):
    _setup(tmp_path, first_signal=3)
    args = [_tool(), str(tmp_path / "run_h.nc"), str(tmp_path / "target.nc"), str(tmp_path / "case"), "m"]
    r = subprocess.run(args, input="", capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "no still sea threshold" in r.stderr


def test_without_a_gpu_the_scan_fails_loudly(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    _setup(tmp_path, first_signal=3)
    r, base = _run(tmp_path, "m")
    assert r.returncode == 1 and "boundary_scan" in r.stderr
    assert not os.path.exists(base + "_west.nc")
