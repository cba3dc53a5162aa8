"""ctypes bindings and a small run driver for the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  The C library is
an FP64 restatement of the reference (cliffs.f, cliffs_main.f time loop,
MasterGrid.f metrics, NestedGrid.f/feed_children_grid.f nesting,
apply_initial_conditions.f, output_*.f conversions).  Its line update is
pinned bit for bit to the reference's own subroutine cliffs, translated from
the checkout's Fortran to C and compiled by oracle/ref_f2c.py
(tests/test_oracle_reference.py); the time loop around it is checked by
reading, and physics-level parity against the analytic profiles of
Examples/slpbeach.zip.

Grids are numpy arrays of shape (ny, nx) in C order, i.e. the Fortran
(nx, ny) column-major layout with x fastest.
"""
import ctypes
import os

import numpy as np

from .build import LIB, LIB32, build

GRAV = 9.800000190734863   # (double)9.8f, global_modules.f:17
PI = 3.1415927410125732    # (double)3.1415926536f
EARTHR = 6371009.0
NAN4 = np.float32(-1.0e32)

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int32)


class OrcGrid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("dep", _dp), ("cel", _dp), ("xvel", _dp), ("yvel", _dp),
                ("hmax", _dp), ("velmax", _dp),
                ("s1", _dp), ("s2", _dp), ("zeta", _dp),
                ("ground", ctypes.c_double), ("crough", ctypes.c_double),
                ("dt", ctypes.c_double), ("celmin", ctypes.c_double),
                ("edge1", _dp), ("edge2", _dp), ("mx", ctypes.c_int32),
                ("xrun", ctypes.c_int32), ("yrun", ctypes.c_int32),
                ("ii1", ctypes.c_int32), ("ii2", ctypes.c_int32),
                ("jj1", ctypes.c_int32), ("jj2", ctypes.c_int32),
                ("seg_overflow", ctypes.c_int32)]


class OrcFeed(ctypes.Structure):
    _fields_ = [("nt", ctypes.c_int32), ("tinput", _dp),
                ("west", _dp), ("east", _dp), ("south", _dp), ("north", _dp),
                ("irec", ctypes.c_int32), ("bndr_input", ctypes.c_int32),
                ("freeze", ctypes.c_int32), ("ended_step", ctypes.c_int32)]


class OrcNest(ctypes.Structure):
    _fields_ = [("mm", ctypes.c_int32), ("nn", ctypes.c_int32),
                ("W_nx", ctypes.c_int32), ("E_nx", ctypes.c_int32),
                ("S_ny", ctypes.c_int32), ("N_ny", ctypes.c_int32),
                ("W_cx", ctypes.c_double), ("E_cx", ctypes.c_double),
                ("S_cy", ctypes.c_double), ("N_cy", ctypes.c_double),
                ("WE_ny", _ip), ("WE_cy", _dp), ("SN_nx", _ip), ("SN_cx", _dp)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        G = ctypes.POINTER(OrcGrid)
        F = ctypes.POINTER(OrcFeed)
        N = ctypes.POINTER(OrcNest)
        L.orc_line.argtypes = [G, ctypes.c_int, ctypes.c_int]
        L.orc_line_local.argtypes = [G, ctypes.c_int, ctypes.c_int]
        L.orc_sweep.argtypes = [G, ctypes.c_int, ctypes.c_int]
        L.orc_maxwave_update.argtypes = [G]
        L.orc_step.argtypes = [G, F, _dp, ctypes.c_int]
        L.orc_step.restype = ctypes.c_int
        L.orc_run.argtypes = [G, F, _dp, ctypes.c_int, ctypes.c_int]
        L.orc_run.restype = ctypes.c_int
        L.orc_wall.argtypes = [_dp, ctypes.c_int64, ctypes.c_double]
        L.orc_celerity.argtypes = [_dp, ctypes.c_int64, ctypes.c_double]
        L.orc_celerity.restype = ctypes.c_double
        L.orc_apply_ic.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                   ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.orc_pinpoint.argtypes = [_dp, ctypes.c_int, ctypes.c_double, _ip, _dp]
        L.orc_depth_ssl.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double, _ip]
        L.orc_depth_ssl.restype = ctypes.c_int
        L.orc_boundary_scan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp, ctypes.c_double]
        L.orc_boundary_scan.restype = ctypes.c_int
        L.orc_boundary_edges.argtypes = [N, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp, ctypes.c_double,
                                         ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_metrics.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  _dp, _dp, _dp, _dp, _dp]
        L.orc_nest_tables.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int,
                                      _dp, ctypes.c_int, _dp, ctypes.c_int, N]
        L.orc_feed_child.argtypes = [G, N, ctypes.c_double, ctypes.c_double,
                                     _ip, _dp, _dp, _dp, _dp]
        L.orc_feed_child.restype = ctypes.c_int
        L.orc_feed_start.argtypes = [F, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.orc_feed_start.restype = ctypes.c_int
        L.orc_maxwave_out.argtypes = [G, _fp, _fp]
        L.orc_sea_state.argtypes = [G, ctypes.c_int, ctypes.c_int, _fp, _fp, _fp]
        L.orc_gauges.argtypes = [G, ctypes.c_int, _ip, _ip, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else ctypes.cast(None, t)


def pinpoint(xx, xp):
    xx = np.ascontiguousarray(xx, dtype=np.float64)
    ip = ctypes.c_int32()
    cp = ctypes.c_double()
    lib().orc_pinpoint(_p(xx), len(xx), float(xp), ctypes.byref(ip), ctypes.byref(cp))
    return ip.value, cp.value


def metrics(xcrd, ycrd, cartesian):
    """MasterGrid.f:85-116 -> (s1 (ny, nx-1) or None, s2 or None, zeta or None)."""
    xcrd = np.ascontiguousarray(xcrd, dtype=np.float64)
    ycrd = np.ascontiguousarray(ycrd, dtype=np.float64)
    nx, ny = len(xcrd), len(ycrd)
    s1 = np.zeros((ny, nx - 1)) if nx > 2 else None
    s2 = np.zeros(ny - 1) if ny > 2 else None
    zeta = np.zeros(ny) if ny > 2 else None
    lib().orc_metrics(nx, ny, int(bool(cartesian)), _p(xcrd), _p(ycrd),
                      _p(s1), _p(s2), _p(zeta))
    return s1, s2, zeta


def apply_ic(xq, yq, qq, xp, yp, pp):
    """apply_initial_conditions.f: pp (ky, kx) += bilinear(qq (ny, nx))."""
    xq = np.ascontiguousarray(xq, dtype=np.float64)
    yq = np.ascontiguousarray(yq, dtype=np.float64)
    qq = np.ascontiguousarray(qq, dtype=np.float64)
    xp = np.ascontiguousarray(xp, dtype=np.float64)
    yp = np.ascontiguousarray(yp, dtype=np.float64)
    assert pp.flags.c_contiguous and pp.dtype == np.float64
    lib().orc_apply_ic(len(xq), len(yq), _p(xq), _p(yq), _p(qq),
                       len(xp), len(yp), _p(xp), _p(yp), _p(pp))


def depth_ssl(dep, alpha=2.0, depmin=0.1):
    """depth_ssl/depth_ssl.f:222-362 (setSSLim) on a copy of dep (ny, nx);
    returns (adjusted depth, per-passage counts (24,), status)."""
    b = np.array(dep, dtype=np.float64, order="C", copy=True)
    counts = np.zeros(24, np.int32)
    ny, nx = b.shape
    st = lib().orc_depth_ssl(nx, ny, _p(b), float(alpha), float(depmin), _p(counts, _ip))
    return b, counts, st


def boundary_scan(cube, cuke):
    """cmpboundary/scan4wave.f on a footprint cube (nt, ny, nx) of float32:
    the first 1-based record above cuke in magnitude, or nt + 1 (the
    reference counts any result >= nt as no signal)."""
    c = np.ascontiguousarray(cube, dtype=np.float32)
    nt, ny, nx = c.shape
    return lib().orc_boundary_scan(nx, ny, nt, _p(c, _fp), float(cuke))


def boundary_edges(tables, cubes, scale=1.0):
    """cmpboundary/InterpolateOntoBndr.f:6-38: the edge records of a target
    grid (NestTables of its coordinates in the source lattice) from the
    footprint cubes (u, v, eta), each (nt, ny, nx) float32.  Returns west,
    east (nt, 3, nn) and south, north (nt, 3, mm)."""
    nt = cubes[0].shape[0]
    mm, nn = tables.mm, tables.nn
    w, e = np.zeros((nt, 3, nn)), np.zeros((nt, 3, nn))
    s, n = np.zeros((nt, 3, mm)), np.zeros((nt, 3, mm))
    for ival, cube in enumerate(cubes, start=1):
        c = np.ascontiguousarray(cube, dtype=np.float32)
        _, ny, nx = c.shape
        lib().orc_boundary_edges(ctypes.byref(tables.s), nx, ny, nt, _p(c, _fp), float(scale), ival,
                                 _p(w), _p(e), _p(s), _p(n))
    return w, e, s, n


class NestTables:
    """NestedGrid.f:104-119 tables for one child grid."""

    def __init__(self, xcrd, ycrd, xnst, ynst):
        xcrd = np.ascontiguousarray(xcrd, dtype=np.float64)
        ycrd = np.ascontiguousarray(ycrd, dtype=np.float64)
        xnst = np.ascontiguousarray(xnst, dtype=np.float64)
        ynst = np.ascontiguousarray(ynst, dtype=np.float64)
        mm, nn = len(xnst), len(ynst)
        self.WE_ny = np.zeros(nn, np.int32)
        self.WE_cy = np.zeros(nn)
        self.SN_nx = np.zeros(mm, np.int32)
        self.SN_cx = np.zeros(mm)
        self.s = OrcNest(mm=mm, nn=nn, WE_ny=_p(self.WE_ny, _ip), WE_cy=_p(self.WE_cy),
                         SN_nx=_p(self.SN_nx, _ip), SN_cx=_p(self.SN_cx))
        lib().orc_nest_tables(_p(xcrd), len(xcrd), _p(ycrd), len(ycrd),
                              _p(xnst), mm, _p(ynst), nn, ctypes.byref(self.s))
        self.mm, self.nn = mm, nn

    def as_dict(self):
        s = self.s
        return dict(W_nx=s.W_nx, E_nx=s.E_nx, S_ny=s.S_ny, N_ny=s.N_ny,
                    W_cx=s.W_cx, E_cx=s.E_cx, S_cy=s.S_cy, N_cy=s.N_cy,
                    WE_ny=self.WE_ny.copy(), WE_cy=self.WE_cy.copy(),
                    SN_nx=self.SN_nx.copy(), SN_cx=self.SN_cx.copy())


class Model:
    """FP64 state of one Cliffs grid and the time loop of cliffs_main.f.

    dep is the still-water depth after wall/deformation; cel is the initial
    total depth H (dep + surface deformation) before the celerity transform of
    cliffs_main.f:218-227, which the constructor applies.
    """

    def __init__(self, dep, s1, s2, zeta, *, ground, crough, dt, cel=None,
                 xvel=None, yvel=None, feed=None, t0=0.0):
        L = lib()
        self.dep = np.ascontiguousarray(dep, dtype=np.float64).copy()
        ny, nx = self.dep.shape
        self.nx, self.ny = nx, ny
        H = self.dep.copy() if cel is None else np.ascontiguousarray(cel, np.float64).copy()
        self.cel = H
        self.celmin = L.orc_celerity(_p(self.cel), self.cel.size, float(ground))
        self.xvel = np.zeros((ny, nx)) if xvel is None else np.ascontiguousarray(xvel, np.float64).copy()
        self.yvel = np.zeros((ny, nx)) if yvel is None else np.ascontiguousarray(yvel, np.float64).copy()
        self.hmax = np.zeros((ny, nx))
        self.velmax = np.zeros((ny, nx))
        self.s1 = None if s1 is None else np.ascontiguousarray(s1, np.float64)
        self.s2 = None if s2 is None else np.ascontiguousarray(s2, np.float64)
        self.zeta = None if zeta is None else np.ascontiguousarray(zeta, np.float64)
        xrun, yrun = nx > 2, ny > 2
        ii1, ii2 = (2, nx - 1) if xrun else (1, 1)
        jj1, jj2 = (2, ny - 1) if yrun else (1, 1)
        self.mx = max(ny if xrun else 1, nx if yrun else 1)
        self.edge1 = np.zeros((3, self.mx))
        self.edge2 = np.zeros((3, self.mx))
        self.g = OrcGrid(nx=nx, ny=ny, dep=_p(self.dep), cel=_p(self.cel),
                         xvel=_p(self.xvel), yvel=_p(self.yvel),
                         hmax=_p(self.hmax), velmax=_p(self.velmax),
                         s1=_p(self.s1), s2=_p(self.s2), zeta=_p(self.zeta),
                         ground=float(ground), crough=float(crough), dt=float(dt),
                         celmin=self.celmin, edge1=_p(self.edge1), edge2=_p(self.edge2),
                         mx=self.mx, xrun=int(xrun), yrun=int(yrun),
                         ii1=ii1, ii2=ii2, jj1=jj1, jj2=jj2, seg_overflow=0)
        self.t = ctypes.c_double(float(t0))
        self.istep = 0
        self.feed = None
        self._feed_arrays = None
        if feed is not None:
            self.set_feed(**feed)

    # -- boundary forcing ------------------------------------------------
    def set_feed(self, tinput, west=None, east=None, south=None, north=None,
                 irec=1, freeze=True):
        """Records in reference layout: west/east (nt, 3, ny), south/north (nt, 3, nx)."""
        arr = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        self._feed_arrays = [arr(tinput), arr(west), arr(east), arr(south), arr(north)]
        t, w, e, s, n = self._feed_arrays
        self.feed = OrcFeed(nt=len(t), tinput=_p(t), west=_p(w), east=_p(e),
                            south=_p(s), north=_p(n), irec=int(irec), bndr_input=1,
                            freeze=int(bool(freeze)), ended_step=0)

    def feed_start(self, cuke):
        g = self.g
        return lib().orc_feed_start(ctypes.byref(self.feed), self.nx, self.ny,
                                    g.xrun, g.yrun, float(cuke))

    # -- stepping ---------------------------------------------------------
    def step(self, nsteps=1):
        """Advance nsteps time steps; returns steps done (fewer if frozen)."""
        f = ctypes.byref(self.feed) if self.feed is not None else ctypes.cast(None, ctypes.POINTER(OrcFeed))
        done = lib().orc_run(ctypes.byref(self.g), f, ctypes.byref(self.t),
                             self.istep + 1, int(nsteps))
        self.istep += done
        return done

    def sweep(self, iu, local=False):
        lib().orc_sweep(ctypes.byref(self.g), int(iu), int(bool(local)))

    def line(self, iu, irw, local=False):
        fn = lib().orc_line_local if local else lib().orc_line
        fn(ctypes.byref(self.g), int(iu), int(irw))

    @property
    def time(self):
        return self.t.value

    @property
    def seg_overflow(self):
        return bool(self.g.seg_overflow)

    # -- outputs ------------------------------------------------------------
    def eta(self):
        e = self.cel * self.cel / GRAV - self.dep
        return np.where(self.cel > self.celmin, e, np.nan)

    def maxwave(self):
        hh = np.zeros((self.ny, self.nx), np.float32)
        vv = np.zeros((self.ny, self.nx), np.float32)
        lib().orc_maxwave_out(ctypes.byref(self.g), _p(hh, _fp), _p(vv, _fp))
        return hh, vv

    def sea_state(self, lonsub=1, latsub=1):
        nxs = (self.nx - 1) // lonsub + 1
        nys = (self.ny - 1) // latsub + 1
        h = np.zeros((nys, nxs), np.float32)
        u = np.zeros((nys, nxs), np.float32)
        v = np.zeros((nys, nxs), np.float32)
        lib().orc_sea_state(ctypes.byref(self.g), lonsub, latsub, _p(h, _fp), _p(u, _fp), _p(v, _fp))
        return h, u, v

    def gauges(self, I, J):
        I = np.ascontiguousarray(I, np.int32)
        J = np.ascontiguousarray(J, np.int32)
        n = len(I)
        eta, u, v = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().orc_gauges(ctypes.byref(self.g), n, _p(I, _ip), _p(J, _ip), _p(eta), _p(u), _p(v))
        return eta, u, v

    def feed_child(self, tables, cuke, iarv):
        """feed_children_grid.f for one child; returns (arrived, (w, e, s, n))."""
        a = ctypes.c_int32(int(bool(iarv)))
        mm, nn = tables.mm, tables.nn
        w, e = np.zeros((3, nn)), np.zeros((3, nn))
        s, n = np.zeros((3, mm)), np.zeros((3, mm))
        r = lib().orc_feed_child(ctypes.byref(self.g), ctypes.byref(tables.s),
                                 float(self.g.ground), float(cuke), ctypes.byref(a),
                                 _p(w), _p(e), _p(s), _p(n))
        if r < 0:
            raise MemoryError("orc_feed_child")
        return bool(a.value), (w, e, s, n) if r == 1 else None


# -- FP32 variant of the time loop (a timed CPU baseline, not a checker) -----

class OrcGrid32(ctypes.Structure):
    """orc_grid of the FP32 build (orc_real = float)."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("dep", _fp), ("cel", _fp), ("xvel", _fp), ("yvel", _fp),
                ("hmax", _fp), ("velmax", _fp),
                ("s1", _fp), ("s2", _fp), ("zeta", _fp),
                ("ground", ctypes.c_float), ("crough", ctypes.c_float),
                ("dt", ctypes.c_float), ("celmin", ctypes.c_float),
                ("edge1", _fp), ("edge2", _fp), ("mx", ctypes.c_int32),
                ("xrun", ctypes.c_int32), ("yrun", ctypes.c_int32),
                ("ii1", ctypes.c_int32), ("ii2", ctypes.c_int32),
                ("jj1", ctypes.c_int32), ("jj2", ctypes.c_int32),
                ("seg_overflow", ctypes.c_int32)]


_lib32 = None


def lib32():
    global _lib32
    if _lib32 is None:
        if not os.path.exists(LIB32):
            build()
        L = ctypes.CDLL(LIB32)
        G = ctypes.POINTER(OrcGrid32)
        L.orc_run.argtypes = [G, ctypes.POINTER(OrcFeed), _dp, ctypes.c_int, ctypes.c_int]
        L.orc_run.restype = ctypes.c_int
        L.orc_celerity.argtypes = [_fp, ctypes.c_int64, ctypes.c_float]
        L.orc_celerity.restype = ctypes.c_float
        _lib32 = L
    return _lib32


class Model32:
    """The time loop of Model in FP32 (the same source built with
    orc_real = float): plain steps without forcing, for timing only."""

    def __init__(self, dep, s1, s2, zeta, *, ground, crough, dt, cel=None, xvel=None, yvel=None):
        L = lib32()
        f32 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32).copy()
        self.dep = f32(dep)
        ny, nx = self.dep.shape
        self.cel = self.dep.copy() if cel is None else f32(cel)
        self.celmin = L.orc_celerity(_p(self.cel, _fp), self.cel.size, float(ground))
        self.xvel = np.zeros((ny, nx), np.float32) if xvel is None else f32(xvel)
        self.yvel = np.zeros((ny, nx), np.float32) if yvel is None else f32(yvel)
        self.hmax = np.zeros((ny, nx), np.float32)
        self.velmax = np.zeros((ny, nx), np.float32)
        self.s1, self.s2, self.zeta = f32(s1), f32(s2), f32(zeta)
        xrun, yrun = nx > 2, ny > 2
        ii1, ii2 = (2, nx - 1) if xrun else (1, 1)
        jj1, jj2 = (2, ny - 1) if yrun else (1, 1)
        mx = max(ny if xrun else 1, nx if yrun else 1)
        self.edge1 = np.zeros((3, mx), np.float32)
        self.edge2 = np.zeros((3, mx), np.float32)
        q = lambda a: _p(a, _fp)
        self.g = OrcGrid32(nx=nx, ny=ny, dep=q(self.dep), cel=q(self.cel), xvel=q(self.xvel), yvel=q(self.yvel),
                           hmax=q(self.hmax), velmax=q(self.velmax), s1=q(self.s1), s2=q(self.s2),
                           zeta=q(self.zeta), ground=float(ground), crough=float(crough), dt=float(dt),
                           celmin=self.celmin, edge1=q(self.edge1), edge2=q(self.edge2), mx=mx,
                           xrun=int(xrun), yrun=int(yrun), ii1=ii1, ii2=ii2, jj1=jj1, jj2=jj2, seg_overflow=0)
        self.t = ctypes.c_double(0.0)
        self.istep = 0

    def step(self, nsteps=1):
        done = lib32().orc_run(ctypes.byref(self.g), ctypes.cast(None, ctypes.POINTER(OrcFeed)),
                               ctypes.byref(self.t), self.istep + 1, int(nsteps))
        self.istep += done
        return done
