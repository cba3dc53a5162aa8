"""Pin the oracle against the reference's only known-answer data.

Examples/slpbeach.zip ships a 1-D bathymetry (a 1:19.85 beach), a solitary
wave of height 0.0185 d as initial state, the run parameters, and analytic
surface profiles at dimensionless times 40, 50, 60 and 70 together with the
MATLAB script that overlays them on the model's screenshots
(plotprofile0185_cliffs_vs_analyt.m).  The reference states no tolerance; the
one chosen here is physics-level: RMS error <= 10 % and max error <= 25 % of
the incident wave height over -2 <= x/d <= 16, the window the script plots.
Measured on this oracle: RMS 4-7 %, max 15-21 %.

The archive is read at test time and not copied into this repository; the
test is skipped on hosts without the reference checkout.
"""
import io
import os
import zipfile

import numpy as np
import pytest

import oracle


def _load(reference_dir):
    zf = zipfile.ZipFile(os.path.join(reference_dir, "Examples", "slpbeach.zip"))
    try:
        from scipy.io import netcdf_file
    except ImportError:  # pragma: no cover
        pytest.skip("scipy not available")

    def nc(name):
        return netcdf_file(io.BytesIO(zf.read("slpbeach/" + name)), "r", mmap=False)

    params = zf.read("slpbeach/slpbeach_params.txt").decode().split("\n")
    vals = [p.split()[0] for p in params if p.strip()]
    # positional parameter file (allabout.f:21-93)
    ground, crough, dt, steps = float(vals[4]), float(vals[5]), float(vals[8]), int(vals[9])
    seaout = int(vals[12])
    b = nc("slpbeach1D.nc")
    x = np.array(b.variables["xxx"][:], np.float64)
    y = np.array(b.variables["yyy"][:], np.float64)
    dep = np.array(b.variables["bathy"][:], np.float64).reshape(len(y), len(x))
    h = nc("solitary.0185_h.nc")
    u = nc("solitary.0185_u.nc")
    xs = np.array(h.variables["xxx"][:], np.float64)
    ys = np.array(h.variables["yyy"][:], np.float64)
    ha = np.array(h.variables["ha"][:], np.float64)[0]
    ua = np.array(u.variables["ua"][:], np.float64)[0]
    ha[ha < -1.0e10] = 0  # get_initial_state.f:153-154
    ua[ua < -1.0e10] = 0
    prof = []
    for line in zf.read("slpbeach/canonical_profiles.txt").decode().strip().splitlines():
        prof.append([float(v) if v != "NaN" else np.nan for v in line.split()])
    return dict(x=x, y=y, dep=dep, xs=xs, ys=ys, ha=ha, ua=ua, ground=ground,
                crough=crough, dt=dt, steps=steps, seaout=seaout, prof=np.array(prof))


def test_slpbeach_analytic_profiles(reference_dir):
    c = _load(reference_dir)
    x, y, dep = c["x"], c["y"], c["dep"]
    s1, s2, zeta = oracle.metrics(x, y, True)
    H = dep.copy()
    U = np.zeros_like(dep)
    oracle.apply_ic(c["xs"], c["ys"], c["ua"], x, y, U)   # cliffs_main.f:199-200
    oracle.apply_ic(c["xs"], c["ys"], c["ha"], x, y, H)   # quake=0: deform surface
    m = oracle.Model(dep, s1, s2, zeta, ground=c["ground"], crough=c["crough"],
                     dt=c["dt"], cel=H, xvel=U)
    d = dep[0, -1]
    A = 0.0185 * d
    anx, anh = c["prof"][:, 0], c["prof"][:, [2, 4, 6, 8]]
    shots = {}
    for k in range(1, c["steps"] + 1):
        m.step(1)
        if k % c["seaout"] == 0:
            shots[k] = m.sea_state()[0][0].astype(np.float64)
        if k * c["dt"] * np.sqrt(9.81 / d) > 72:
            break
    ks = np.array(sorted(shots))
    tt = np.sqrt(9.81 / d) * ks * c["dt"]   # plotprofile0185_cliffs_vs_analyt.m
    for i, ts in enumerate([40, 50, 60, 70]):
        k = ks[np.argmin(abs(tt - ts))]
        hh = shots[k]
        hh[hh < -9999] = np.nan
        model = np.interp(anx, x, hh)
        ok = ~np.isnan(anh[:, i]) & ~np.isnan(model) & (anx >= -2) & (anx <= 16)
        err = model[ok] - anh[ok, i] * d
        assert ok.sum() > 100
        assert np.sqrt(np.mean(err ** 2)) <= 0.10 * A, (ts, np.sqrt(np.mean(err ** 2)))
        assert np.abs(err).max() <= 0.25 * A, (ts, np.abs(err).max())
