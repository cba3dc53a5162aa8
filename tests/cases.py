"""Synthetic Cliffs runs in the reference's file formats, for the driver tests.

write_case() lays out what the reference's executable reads:
  <dir>/params.txt                  allabout.f's positional parameter file
  <dir>/master.nc                   MasterGrid.f: x, y, depth (float)
  <dir>/child.nc                    NestedGrid.f: a child grid's x, y
  <dir>/src_h.nc (and _u)           get_initial_state.f: one record on a coarse lattice
  <dir>/bnd_master_{west,...}.nc    get_boundary_feed.f: (u, v, eta) edge records
NetCDF files are written with scipy.io.netcdf_file (NetCDF-3 classic), an
implementation independent of the driver's own.  reference_setup() restates
the same setup with the oracle (apply_initial_conditions, wall, deformation,
nest tables, feed start) so the driver can be checked against it.
"""
import importlib
import os

import numpy as np
from scipy.io import netcdf_file

import oracle

W = importlib.import_module("cliffs-src_gb300").workloads


def _nc_grid(path, x, y, z, zname="bathy"):
    f = netcdf_file(path, "w")
    f.createDimension("xxx", len(x))
    f.createDimension("yyy", len(y))
    vx = f.createVariable("xxx", "d", ("xxx",))
    vy = f.createVariable("yyy", "d", ("yyy",))
    vz = f.createVariable(zname, "f", ("yyy", "xxx"))
    vx[:] = x
    vy[:] = y
    vz[:] = z
    f.close()


def _nc_field(path, name, x, y, t, vals):
    f = netcdf_file(path, "w")
    f.createDimension("time", None)
    f.createDimension("xxx", len(x))
    f.createDimension("yyy", len(y))
    vx = f.createVariable("xxx", "d", ("xxx",))
    vy = f.createVariable("yyy", "d", ("yyy",))
    vt = f.createVariable("time", "d", ("time",))
    vv = f.createVariable(name, "f", ("time", "yyy", "xxx"))
    vx[:] = x
    vy[:] = y
    vt[:] = t
    vv[:] = vals
    f.close()


def _nc_feed(path, recs, t):
    """recs (nt, 3, len): the layout of opennc4feed.f (pnt, uvq, tim)."""
    f = netcdf_file(path, "w")
    f.createDimension("tim", None)  # scipy wants the record dimension defined first
    f.createDimension("pnt", recs.shape[2])
    f.createDimension("uvq", 3)
    vv = f.createVariable("vals", "d", ("tim", "uvq", "pnt"))
    vt = f.createVariable("time", "d", ("tim",))
    vv[:] = recs
    vt[:] = t
    f.close()


def write_case(d, *, nx=192, ny=160, dx=1000.0, seed=3, steps=240, seaout=80, gout=20, maxout=120,
               bndout=20, ngauges=6, child=True, feed=True, source=True, quake=1, itopo=1, dwall=2.0,
               freeze=False, crough=0.000625, amp=1.5):
    """Write one run into directory d; returns a dict of what was written."""
    os.makedirs(d, exist_ok=True)
    case = W.shelf_2d(seed=seed, nx=nx, ny=ny, dx=dx, steps=0, amp=0.0, ngauges=ngauges)
    x, y, dep = case["xcrd"], case["ycrd"], case["dep"].astype(np.float32)
    _nc_grid(os.path.join(d, "master.nc"), x, y, dep)
    out = dict(x=x, y=y, dep=dep.astype(np.float64), dt=case["dt"], ground=case["ground"],
               crough=crough, steps=steps, seaout=seaout, gout=gout, maxout=maxout, bndout=bndout,
               quake=quake, itopo=itopo, dwall=dwall, freeze=freeze)
    lines = ["1\t(1 - cartesian, otherwise-spherical)", "master.nc"]
    if child:
        xn = np.arange(x[60] + 150.0, x[130], dx / 3)
        yn = np.arange(y[40] + 90.0, y[110], dx / 3)
        _nc_grid(os.path.join(d, "child.nc"), xn, yn, np.zeros((len(yn), len(xn)), np.float32))
        out.update(xn=xn, yn=yn)
        lines += ["1\tNumber of grids enclosed in Master", "child.nc"]
    else:
        lines += ["0\tNumber of grids enclosed in Master"]
    I, J = case["gauges"]
    lines += ["0.001\tStill sea threshold on the boundary (m)",
              f"{case['ground']}\tMinimal flow depth (m)",
              f"{crough}\tfriction coefficient (Manning n**2)",
              f"{itopo}\ttopo flag: 0-wall, otherwise - land inundation",
              f"{dwall}\tVertical wall, if any, at depth (m)",
              f"{case['dt']!r}\ttime step (sec)",
              f"{steps}\ttotal amount of steps",
              f"{quake}\t1 - to deform bottom",
              f"{0 if freeze else 1}\t0 - to stop when boundary forcing stops",
              f"{seaout}\tsteps between screenshots",
              "2\tsubsample screenshots in x",
              "3\tsubsample screenshots in y",
              f"{bndout}\tsave feed into nested grids every n steps",
              f"{maxout}\tsteps between maxwave updates",
              f"{ngauges}\tN gages"]
    if ngauges:
        lines.append(f"{gout}")
        lines += [f"{i} {j}" for i, j in zip(I, J)]
    out.update(I=np.asarray(I, np.int32), J=np.asarray(J, np.int32), lonsub=2, latsub=3)
    with open(os.path.join(d, "params.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    rng = np.random.default_rng(seed)
    if source:
        # an elliptical uplift on a coarse lattice covering part of the grid
        xs = np.linspace(x[20], x[110], 46)
        ys = np.linspace(y[30], y[130], 51)
        X, Y = np.meshgrid(xs, ys)
        q = amp * np.exp(-((X - x[60]) / 25e3) ** 2 - ((Y - y[80]) / 15e3) ** 2)
        tsrc = np.array([0.0, 600.0])
        vals = np.stack([q, 0.5 * q]).astype(np.float32)
        _nc_field(os.path.join(d, "src_h.nc"), "ha", xs, ys, tsrc, vals)
        uvals = np.stack([0.01 * q, 0.02 * q]).astype(np.float32)
        _nc_field(os.path.join(d, "src_u.nc"), "ua", xs, ys, tsrc, uvals)
        out.update(xs=xs, ys=ys, q=vals.astype(np.float64), qu=uvals.astype(np.float64), tsrc=tsrc)
    if feed:
        nt = 40
        tin = np.arange(nt) * 6 * case["dt"]
        recs = {}
        for side, length, ph in (("west", ny, 0.0), ("east", ny, 0.3), ("south", nx, 0.1), ("north", nx, 0.6)):
            r = np.zeros((nt, 3, length))
            s = np.linspace(0, 1, length)
            for k in range(nt):
                w = 0.2 * np.sin(2 * np.pi * (tin[k] / 400.0 + ph)) * (0.5 + 0.5 * np.cos(np.pi * s))
                r[k, 2] = w if k >= 3 else 0.0
                r[k, 0] = 0.1 * r[k, 2]
                r[k, 1] = 0.02 * r[k, 2]
            recs[side] = r
            _nc_feed(os.path.join(d, f"bnd_master_{side}.nc"), r, tin)
        out.update(tinput=tin, **recs)
    return out


def reference_setup(c, *, aprfx=True, bprfx=True, cuke=0.001):
    """The setup of cliffs_main.f:131-227 on the oracle for a written case:
    dep after wall and deformation, H before the celerity transform, u, v,
    the start record and time."""
    dep = c["dep"].copy()
    if c["itopo"] == 0:
        dep[dep <= c["dwall"]] = -999.0
    H = dep.copy()
    u = np.zeros_like(dep)
    v = np.zeros_like(dep)
    irec, t0 = 1, 0.0
    m0 = None
    if bprfx:
        s1, s2, zeta = oracle.metrics(c["x"], c["y"], True)
        m0 = oracle.Model(dep, s1, s2, zeta, ground=c["ground"], crough=c["crough"], dt=c["dt"])
        m0.set_feed(c["tinput"], c["west"], c["east"], c["south"], c["north"], irec=1, freeze=c["freeze"])
        irec = m0.feed_start(cuke)
        t0 = float(c["tinput"][irec - 1])
    if aprfx:
        if bprfx:
            ip, _ = oracle.pinpoint(c["tsrc"], t0)
            isrc = ip
        else:
            isrc, t0 = 1, float(c["tsrc"][0])
        oracle.apply_ic(c["xs"], c["ys"], c["qu"][isrc - 1], c["x"], c["y"], u)
        q = c["q"][isrc - 1]
        if c["quake"] == 1:
            oracle.apply_ic(c["xs"], c["ys"], -q, c["x"], c["y"], dep)
        else:
            oracle.apply_ic(c["xs"], c["ys"], q, c["x"], c["y"], H)
    return dict(dep=dep, H=H, u=u, v=v, irec=irec, t0=t0)
