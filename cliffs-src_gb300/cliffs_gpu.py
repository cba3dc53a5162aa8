"""Python binding of the C ABI in include/cliffs_gpu.h (ctypes).

GpuGrid mirrors the state a Cliffs run keeps in module MASTER
(global_modules.f:16-35) and the operations the time loop of
cliffs_main.f:303-378 applies to it.  Every compute call goes to the CUDA
library; there is no CPU path, and loading fails loudly when the library is
missing.  Arrays are numpy arrays of shape (ny, nx), C order, which is the
Fortran (nx, ny) column-major layout.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcliffs_gpu.so")

CLIFFS_OK = 0
CLIFFS_FEED_ENDED = 1
CLIFFS_WARN_CFL = 2
CLIFFS_ST_NAN, CLIFFS_ST_STALL, CLIFFS_ST_CFL = 1, 2, 4
GRAV = 9.800000190734863

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int32)


class GridDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("dep", _dp),
                ("dx", _dp), ("row_scale", _dp), ("dy", _dp), ("zeta", _dp),
                ("ground", ctypes.c_double), ("crough", ctypes.c_double),
                ("dt", ctypes.c_double)]


class NestDesc(ctypes.Structure):
    _fields_ = [("mm", ctypes.c_int32), ("nn", ctypes.c_int32),
                ("W_nx", ctypes.c_int32), ("E_nx", ctypes.c_int32),
                ("S_ny", ctypes.c_int32), ("N_ny", ctypes.c_int32),
                ("W_cx", ctypes.c_double), ("E_cx", ctypes.c_double),
                ("S_cy", ctypes.c_double), ("N_cy", ctypes.c_double),
                ("WE_ny", _ip), ("WE_cy", _dp), ("SN_nx", _ip), ("SN_cx", _dp)]


class Runup(ctypes.Structure):
    _fields_ = [("max_runup", ctypes.c_double), ("i", ctypes.c_int32),
                ("j", ctypes.c_int32), ("wetted_land", ctypes.c_int64),
                ("wet_now", ctypes.c_int64)]


class SourceDesc(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_double), ("y0", ctypes.c_double), ("ax", ctypes.c_double),
                ("ay", ctypes.c_double), ("angle", ctypes.c_double), ("amp", ctypes.c_double),
                ("dipole", ctypes.c_double), ("rise_time", ctypes.c_double), ("bottom", ctypes.c_int32)]


def source_field(x, y, *, x0, y0, ax, ay, angle=0.0, amp=1.0, dipole=0.0):
    """The uplift of cliffs_gpu_add_source on the grid (ny, nx), in numpy FP64."""
    X, Y = np.meshgrid(np.asarray(x, np.float64), np.asarray(y, np.float64))
    dx, dy = X - x0, Y - y0
    ca, sa = np.cos(angle), np.sin(angle)
    xi, et = ca * dx + sa * dy, -sa * dx + ca * dy
    a, b, b2 = xi / ax, et / ay, (et + 2.0 * ay) / ay
    return amp * (np.exp(-(a * a + b * b)) - dipole * np.exp(-(a * a + b2 * b2)))


class BatchPlan(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("graph_steps", ctypes.c_int32), ("x_rows", ctypes.c_int32), ("y_groups", ctypes.c_int32)]


PERSISTENT, GRAPH = 0, 1
TILED, STAGED, DIRECT = 0, 1, 2  # cliffs_gpu_set_sweep_kernel
LATTICE_SURFACE, LATTICE_BOTTOM, LATTICE_XVEL, LATTICE_YVEL = 0, 1, 2, 3  # cliffs_gpu_apply_lattice


def depth_ssl(dep, alpha=2.0, depmin=0.1):
    """The depth_ssl tool's limiter (cliffs_depth_ssl) on a copy of dep
    (ny, nx); returns (adjusted depth, per-passage counts (24,), status)."""
    b = np.array(dep, dtype=np.float64, order="C", copy=True)
    counts = np.zeros(24, np.int32)
    st = ctypes.c_int32()
    ny, nx = b.shape
    _chk(load().cliffs_depth_ssl(nx, ny, _p(b), float(alpha), float(depmin), _p(counts, _ip), ctypes.byref(st)),
         "depth_ssl")
    return b, counts, st.value


def _nest_desc(t):
    """A cliffs_nest_desc of a tables dict; returns it with the arrays it points to."""
    keep = [np.ascontiguousarray(t["WE_ny"], np.int32), _f64(t["WE_cy"]), np.ascontiguousarray(t["SN_nx"], np.int32),
            _f64(t["SN_cx"])]
    d = NestDesc(mm=len(keep[2]), nn=len(keep[0]), W_nx=int(t["W_nx"]), E_nx=int(t["E_nx"]), S_ny=int(t["S_ny"]),
                 N_ny=int(t["N_ny"]), W_cx=float(t["W_cx"]), E_cx=float(t["E_cx"]), S_cy=float(t["S_cy"]),
                 N_cy=float(t["N_cy"]), WE_ny=_p(keep[0], _ip), WE_cy=_p(keep[1]), SN_nx=_p(keep[2], _ip),
                 SN_cx=_p(keep[3]))
    return d, keep


def boundary_scan(cube, cuke):
    """scan4wave.f on the device (cliffs_boundary_scan): cube (nt, ny, nx)
    float32, the target's footprint; the first 1-based record above cuke in
    magnitude, or nt + 1 (any result >= nt is no signal)."""
    c = np.ascontiguousarray(cube, np.float32)
    nt, ny, nx = c.shape
    first = ctypes.c_int32()
    _chk(load().cliffs_boundary_scan(nx, ny, nt, _p(c, _fp), float(cuke), ctypes.byref(first)), "boundary_scan")
    return first.value


def boundary_edges(tables, cubes, scale=1.0):
    """InterpolateOntoBndr.f on the device (cliffs_boundary_edges): the edge
    records of a target grid from the footprint cubes (u, v, eta), each
    (nt, ny, nx) float32.  Returns west, east (nt, 3, nn), south, north
    (nt, 3, mm)."""
    d, keep = _nest_desc(tables)
    nt = cubes[0].shape[0]
    mm, nn = d.mm, d.nn
    w, e = np.zeros((nt, 3, nn)), np.zeros((nt, 3, nn))
    s, n = np.zeros((nt, 3, mm)), np.zeros((nt, 3, mm))
    for ival, cube in enumerate(cubes, start=1):
        c = np.ascontiguousarray(cube, np.float32)
        _, ny, nx = c.shape
        _chk(load().cliffs_boundary_edges(ctypes.byref(d), nx, ny, nt, _p(c, _fp), float(scale), ival, _p(w), _p(e),
                                          _p(s), _p(n)), "boundary_edges")
    return w, e, s, n


class _Pinned:
    """Owner of one pinned host allocation (cliffs_gpu_host_alloc), freed
    when the last array viewing it goes."""

    def __init__(self, nbytes):
        self.L = load()
        self.ptr = ctypes.c_void_p()
        _chk(self.L.cliffs_gpu_host_alloc(max(nbytes, 1), ctypes.byref(self.ptr)), "host_alloc")

    def __del__(self):
        try:
            if self.ptr:
                self.L.cliffs_gpu_host_free(self.ptr)
        except Exception:
            pass


def pinned(shape, dtype=np.float64):
    """A numpy array in pinned host memory, for the asynchronous outputs."""
    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    owner = _Pinned(count * dtype.itemsize)
    buf = (ctypes.c_char * max(count * dtype.itemsize, 1)).from_address(owner.ptr.value)
    buf._owner = owner  # the array's base keeps the allocation alive
    return np.frombuffer(buf, dtype=dtype, count=count).reshape(shape)


class CliffsError(RuntimeError):
    def __init__(self, code, what):
        self.code = code
        super().__init__(f"{what}: {strerror(code)} ({code})")


# Every symbol declared in include/cliffs_gpu.h with its ctypes signature.
_V = ctypes.c_void_p
_I = ctypes.c_int32
_D = ctypes.c_double
SIGNATURES = {
    "cliffs_gpu_metrics": ([_I, _I, _I, _dp, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_create": ([ctypes.POINTER(GridDesc), ctypes.POINTER(_V)], ctypes.c_int),
    "cliffs_gpu_destroy": ([_V], None),
    "cliffs_gpu_set_stream": ([_V, _V], ctypes.c_int),
    "cliffs_gpu_set_initial": ([_V, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_upload_state": ([_V, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_download_state": ([_V, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_set_feed": ([_V, _I, _dp, _dp, _dp, _dp, _dp, _I, _I], ctypes.c_int),
    "cliffs_gpu_feed_start": ([_V, _D], ctypes.c_int),
    "cliffs_gpu_step": ([_V, _I, _dp, _ip], ctypes.c_int),
    "cliffs_gpu_sweep": ([_V, _I], ctypes.c_int),
    "cliffs_gpu_set_edges": ([_V, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_maxwave_update": ([_V], ctypes.c_int),
    "cliffs_gpu_get_maxwave": ([_V, _fp, _fp], ctypes.c_int),
    "cliffs_gpu_get_max_raw": ([_V, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_get_sea_state": ([_V, _I, _I, _fp, _fp, _fp], ctypes.c_int),
    "cliffs_gpu_get_gauges": ([_V, _I, _ip, _ip, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_runup": ([_V, ctypes.POINTER(Runup)], ctypes.c_int),
    "cliffs_gpu_nest_add": ([_V, ctypes.POINTER(NestDesc), _ip], ctypes.c_int),
    "cliffs_gpu_feed_child": ([_V, _I, _D, _ip, _dp, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_gpu_get_sea_state_async": ([_V, _I, _I, _fp, _fp, _fp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cliffs_gpu_get_gauges_async": ([_V, _I, _ip, _ip, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int64)],
                                    ctypes.c_int),
    "cliffs_gpu_feed_child_async": ([_V, _I, _D, _ip, _dp, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int64)],
                                    ctypes.c_int),
    "cliffs_gpu_output_wait": ([_V, ctypes.c_int64], ctypes.c_int),
    "cliffs_gpu_output_done": ([_V, ctypes.c_int64, _ip], ctypes.c_int),
    "cliffs_gpu_host_alloc": ([ctypes.c_int64, ctypes.POINTER(_V)], ctypes.c_int),
    "cliffs_gpu_host_free": ([_V], None),
    "cliffs_gpu_status": ([_V, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "cliffs_gpu_sync": ([_V], ctypes.c_int),
    "cliffs_gpu_profile": ([_V, _I], ctypes.c_int),
    "cliffs_gpu_profile_read": ([_V, _dp, ctypes.POINTER(ctypes.c_int64), _dp,
                                 ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cliffs_gpu_launch_count": ([_V, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cliffs_gpu_set_graph_steps": ([_V, _I], ctypes.c_int),
    "cliffs_gpu_prepare_steps": ([_V, _I], ctypes.c_int),
    "cliffs_gpu_courant": ([_V, _dp], ctypes.c_int),
    "cliffs_gpu_set_tiling": ([_V, _I, _I], ctypes.c_int),
    "cliffs_gpu_set_sweep_kernel": ([_V, _I], ctypes.c_int),
    "cliffs_gpu_check_stage_timeout": ([_V, _I], ctypes.c_int),
    "cliffs_gpu_strerror": ([ctypes.c_int], ctypes.c_char_p),
    "cliffs_depth_ssl": ([_I, _I, _dp, _D, _D, _ip, _ip], ctypes.c_int),
    "cliffs_boundary_scan": ([_I, _I, _I, _fp, _D, _ip], ctypes.c_int),
    "cliffs_boundary_edges": ([ctypes.POINTER(NestDesc), _I, _I, _I, _fp, _D, _I, _dp, _dp, _dp, _dp],
                              ctypes.c_int),
    "cliffs_gpu_add_source": ([_V, _dp, _dp, ctypes.POINTER(SourceDesc)], ctypes.c_int),
    "cliffs_gpu_apply_lattice": ([_V, _dp, _dp, _I, _I, _dp, _dp, _dp, _I], ctypes.c_int),
    "cliffs_batch_create": ([ctypes.POINTER(_V), _I, ctypes.POINTER(_V)], ctypes.c_int),
    "cliffs_batch_destroy": ([_V], None),
    "cliffs_batch_set_plan": ([_V, ctypes.POINTER(BatchPlan)], ctypes.c_int),
    "cliffs_batch_get_plan": ([_V, ctypes.POINTER(BatchPlan)], ctypes.c_int),
    "cliffs_batch_step": ([_V, _I], ctypes.c_int),
    "cliffs_batch_autotune": ([_V, _I, _dp], ctypes.c_int),
    "cliffs_batch_check_barrier_timeout": ([_V, _I], ctypes.c_int),
    "cliffs_batch_launch_count": ([_V, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cliffs_batch_set_gauges": ([_V, _ip, _ip, _ip], ctypes.c_int),
    "cliffs_batch_get_gauges": ([_V, _dp, _dp, _dp], ctypes.c_int),
    "cliffs_mlp_create": ([ctypes.c_void_p, ctypes.POINTER(_V)], ctypes.c_int),
    "cliffs_mlp_destroy": ([_V], None),
    "cliffs_mlp_layers": ([_V, ctypes.POINTER(_I)], ctypes.c_int),
    "cliffs_mlp_shape": ([_V, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], ctypes.c_int),
    "cliffs_mlp_get": ([_V, _I, _I, ctypes.POINTER(ctypes.c_float), ctypes.c_int64], ctypes.c_int),
    "cliffs_mlp_set": ([_V, _I, _I, ctypes.POINTER(ctypes.c_float), ctypes.c_int64], ctypes.c_int),
    "cliffs_mlp_predict": ([_V, _I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "cliffs_mlp_gradients": ([_V, _I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                              ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "cliffs_mlp_train": ([_V, _I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), _I, _I,
                          ctypes.c_float, ctypes.c_float, ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)],
                         ctypes.c_int),
    "cliffs_mlp_launch_count": ([_V, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cliffs_gpu_sweep_noalloc": ([_I, _I, _I, _I] + [_V] * 7 + [_D] * 5 + [_V], ctypes.c_int),
    "cliffs_gpu_sweep_noalloc_status": ([_V, _V, _V], ctypes.c_int),
}

_lib = None


def load(path=None):
    """Load the CUDA library; raises when it was not built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library not built: {p} (run the package's build.py)")
    L = ctypes.CDLL(p)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    if path is None:
        _lib = L
    return L


def strerror(code):
    try:
        return load().cliffs_gpu_strerror(int(code)).decode()
    except Exception:  # pragma: no cover - library absent
        return "unknown"


def _chk(code, what):
    if code < 0:
        raise CliffsError(code, what)
    return code


def _p(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else ctypes.cast(None, t)


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def metrics(xcrd, ycrd, cartesian):
    """MasterGrid.f:85-116 through the library: (dx, row_scale, dy, zeta)."""
    xcrd = _f64(xcrd)
    ycrd = _f64(ycrd)
    nx, ny = len(xcrd), len(ycrd)
    dx = np.zeros(max(nx - 1, 1))
    rs = np.ones(ny)
    dy = np.zeros(max(ny - 1, 1))
    zeta = np.zeros(ny)
    _chk(load().cliffs_gpu_metrics(nx, ny, int(bool(cartesian)), _p(xcrd), _p(ycrd),
                                   _p(dx), _p(rs), _p(dy), _p(zeta)), "metrics")
    return (dx if nx > 2 else None, rs if nx > 2 and not cartesian else None,
            dy if ny > 2 else None, zeta if ny > 2 else None)


class GpuGrid:
    """Device-resident state of one Cliffs grid."""

    def __init__(self, dep, *, dx=None, row_scale=None, dy=None, zeta=None,
                 ground, crough, dt):
        self.L = load()
        self.dep = _f64(dep)
        self.ny, self.nx = self.dep.shape
        self._keep = [_f64(dx), _f64(row_scale), _f64(dy), _f64(zeta)]
        kdx, krs, kdy, kz = self._keep
        d = GridDesc(nx=self.nx, ny=self.ny, dep=_p(self.dep), dx=_p(kdx),
                     row_scale=_p(krs), dy=_p(kdy), zeta=_p(kz),
                     ground=float(ground), crough=float(crough), dt=float(dt))
        h = ctypes.c_void_p()
        _chk(self.L.cliffs_gpu_create(ctypes.byref(d), ctypes.byref(h)), "create")
        self.h = h
        self.ground, self.crough, self.dt = float(ground), float(crough), float(dt)
        self.celmin = float(np.sqrt(GRAV * self.ground))
        self.t = ctypes.c_double(0.0)
        self._streamref = None

    @classmethod
    def from_case(cls, case):
        dx, rs, dy, zeta = metrics(case["xcrd"], case["ycrd"], case["cartesian"])
        if case.get("zeta") is not None:
            zeta = case["zeta"]
        g = cls(case["dep"], dx=dx, row_scale=rs, dy=dy, zeta=zeta,
                ground=case["ground"], crough=case["crough"], dt=case["dt"])
        g.set_initial(case["H0"], case.get("u0"), case.get("v0"))
        g.t.value = float(case.get("t0", 0.0))
        return g

    def close(self):
        if getattr(self, "h", None):
            self.L.cliffs_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state --------------------------------------------------------------
    def set_stream(self, stream_ptr):
        _chk(self.L.cliffs_gpu_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def set_initial(self, H, u=None, v=None):
        s = (self.ny, self.nx)
        _chk(self.L.cliffs_gpu_set_initial(self.h, _p(_f64(H, s)), _p(_f64(u, s)), _p(_f64(v, s))),
             "set_initial")

    def upload_state(self, cel, u=None, v=None):
        s = (self.ny, self.nx)
        _chk(self.L.cliffs_gpu_upload_state(self.h, _p(_f64(cel, s)), _p(_f64(u, s)), _p(_f64(v, s))),
             "upload_state")

    def _out(self, out, k, dtype):
        if out is None:
            return np.empty((self.ny, self.nx), dtype)
        a = out[k]
        if a.shape != (self.ny, self.nx) or a.dtype != dtype or not a.flags.c_contiguous:
            raise ValueError(f"output {k}: expected C-contiguous {dtype} of shape {(self.ny, self.nx)}")
        return a

    def download_state(self, out=None):
        """(cel, u, v) in FP64; out: three arrays to fill instead of new ones
        (a caller's own arrays, as the Fortran driver keeps them)."""
        cel, u, v = (self._out(out, k, np.float64) for k in range(3))
        _chk(self.L.cliffs_gpu_download_state(self.h, _p(cel), _p(u), _p(v)), "download_state")
        return cel, u, v

    def eta(self):
        cel, _, _ = self.download_state()
        H = cel * np.abs(cel) / GRAV
        return np.where(cel > self.celmin, H - self.dep, np.nan)

    # -- forcing --------------------------------------------------------------
    def add_source(self, x, y, *, x0, y0, ax, ay, angle=0.0, amp=1.0, dipole=0.0, rise_time=0.0,
                   bottom=False):
        """An analytic uplift (cliffs_gpu_add_source) on grid coordinates x, y."""
        d = SourceDesc(float(x0), float(y0), float(ax), float(ay), float(angle), float(amp),
                       float(dipole), float(rise_time), int(bool(bottom)))
        _chk(self.L.cliffs_gpu_add_source(self.h, _p(_f64(x)), _p(_f64(y)), ctypes.byref(d)),
             "add_source")

    def apply_lattice(self, x, y, xq, yq, q, target):
        """apply_initial_conditions.f on the device (cliffs_gpu_apply_lattice):
        lattice q (len(yq), len(xq)) at xq, yq added to target (LATTICE_*)."""
        q = _f64(q)
        xq = _f64(np.atleast_1d(xq))
        yq = _f64(np.atleast_1d(yq))
        _chk(self.L.cliffs_gpu_apply_lattice(self.h, _p(_f64(x)), _p(_f64(y)), len(xq), len(yq), _p(xq), _p(yq),
                                             _p(q), int(target)), "apply_lattice")

    def set_feed(self, tinput, west=None, east=None, south=None, north=None, irec=1, freeze=True):
        arr = [_f64(a) for a in (tinput, west, east, south, north)]
        self._feed = arr
        t, w, e, s, n = arr
        _chk(self.L.cliffs_gpu_set_feed(self.h, len(t), _p(t), _p(w), _p(e), _p(s), _p(n),
                                        int(irec), int(bool(freeze))), "set_feed")

    def feed_start(self, cuke):
        return self.L.cliffs_gpu_feed_start(self.h, float(cuke))

    def set_edges(self, edge1=None, edge2=None):
        e1 = _f64(edge1)
        e2 = _f64(edge2)
        _chk(self.L.cliffs_gpu_set_edges(self.h, _p(e1), _p(e2)), "set_edges")

    # -- stepping -------------------------------------------------------------
    def step(self, nsteps=1):
        done = ctypes.c_int32(0)
        r = _chk(self.L.cliffs_gpu_step(self.h, int(nsteps), ctypes.byref(self.t), ctypes.byref(done)), "step")
        return done.value, r == CLIFFS_FEED_ENDED

    @property
    def time(self):
        return self.t.value

    def sweep(self, iu):
        _chk(self.L.cliffs_gpu_sweep(self.h, int(iu)), "sweep")

    def maxwave_update(self):
        _chk(self.L.cliffs_gpu_maxwave_update(self.h), "maxwave_update")

    def sync(self):
        _chk(self.L.cliffs_gpu_sync(self.h), "sync")

    def status(self):
        f = ctypes.c_uint32(0)
        r = self.L.cliffs_gpu_status(self.h, ctypes.byref(f))
        return r, f.value

    def courant(self):
        """The largest Courant number above 1 any sweep has read (0: none)."""
        x = ctypes.c_double(0.0)
        _chk(self.L.cliffs_gpu_courant(self.h, ctypes.byref(x)), "courant")
        return x.value

    # -- outputs ----------------------------------------------------------------
    def maxwave(self, out=None):
        """(MaxE, MaxV) as output_maxwave.f writes them; out: two float32
        arrays to fill instead of new ones."""
        me, mv = (self._out(out, k, np.float32) for k in range(2))
        _chk(self.L.cliffs_gpu_get_maxwave(self.h, _p(me, _fp), _p(mv, _fp)), "get_maxwave")
        return me, mv

    def max_raw(self):
        hm = np.empty((self.ny, self.nx))
        vm = np.empty((self.ny, self.nx))
        _chk(self.L.cliffs_gpu_get_max_raw(self.h, _p(hm), _p(vm)), "get_max_raw")
        return hm, vm

    def sea_state(self, lonsub=1, latsub=1):
        nxs = (self.nx - 1) // lonsub + 1
        nys = (self.ny - 1) // latsub + 1
        h = np.empty((nys, nxs), np.float32)
        u = np.empty((nys, nxs), np.float32)
        v = np.empty((nys, nxs), np.float32)
        _chk(self.L.cliffs_gpu_get_sea_state(self.h, lonsub, latsub, _p(h, _fp), _p(u, _fp), _p(v, _fp)),
             "get_sea_state")
        return h, u, v

    def gauges(self, I, J):
        I = np.ascontiguousarray(I, np.int32)
        J = np.ascontiguousarray(J, np.int32)
        n = len(I)
        eta, u, v = np.empty(n), np.empty(n), np.empty(n)
        _chk(self.L.cliffs_gpu_get_gauges(self.h, n, _p(I, _ip), _p(J, _ip), _p(eta), _p(u), _p(v)),
             "get_gauges")
        return eta, u, v

    def runup(self):
        r = Runup()
        _chk(self.L.cliffs_gpu_runup(self.h, ctypes.byref(r)), "runup")
        return dict(max_runup=r.max_runup, i=r.i, j=r.j, wetted_land=r.wetted_land, wet_now=r.wet_now)

    # -- nesting ---------------------------------------------------------------
    def nest_add(self, tables):
        """tables: dict with the NestedGrid.f:104-119 fields (1-based)."""
        WE_ny = np.ascontiguousarray(tables["WE_ny"], np.int32)
        WE_cy = _f64(tables["WE_cy"])
        SN_nx = np.ascontiguousarray(tables["SN_nx"], np.int32)
        SN_cx = _f64(tables["SN_cx"])
        d = NestDesc(mm=len(SN_nx), nn=len(WE_ny), W_nx=int(tables["W_nx"]), E_nx=int(tables["E_nx"]),
                     S_ny=int(tables["S_ny"]), N_ny=int(tables["N_ny"]), W_cx=float(tables["W_cx"]),
                     E_cx=float(tables["E_cx"]), S_cy=float(tables["S_cy"]), N_cy=float(tables["N_cy"]),
                     WE_ny=_p(WE_ny, _ip), WE_cy=_p(WE_cy), SN_nx=_p(SN_nx, _ip), SN_cx=_p(SN_cx))
        i = ctypes.c_int32(-1)
        _chk(self.L.cliffs_gpu_nest_add(self.h, ctypes.byref(d), ctypes.byref(i)), "nest_add")
        return i.value, (len(SN_nx), len(WE_ny))

    def feed_child(self, nest, cuke, arrived):
        nid, (mm, nn) = nest
        a = ctypes.c_int32(int(bool(arrived)))
        w, e = np.zeros((3, nn)), np.zeros((3, nn))
        s, n = np.zeros((3, mm)), np.zeros((3, mm))
        r = _chk(self.L.cliffs_gpu_feed_child(self.h, nid, float(cuke), ctypes.byref(a),
                                              _p(w), _p(e), _p(s), _p(n)), "feed_child")
        return bool(a.value), ((w, e, s, n) if r == 1 else None)

    # -- asynchronous outputs --------------------------------------------------------
    def sea_state_async(self, lonsub, latsub, out):
        """Queue a screenshot into out = (h, u, v), float32 arrays (pinned:
        pinned()); returns the ticket for wait()."""
        h, u, v = out
        t = ctypes.c_int64()
        _chk(self.L.cliffs_gpu_get_sea_state_async(self.h, int(lonsub), int(latsub), _p(h, _fp), _p(u, _fp),
                                                   _p(v, _fp), ctypes.byref(t)), "get_sea_state_async")
        return t.value

    def gauges_async(self, I, J, out):
        """Queue a gauge record into out = (eta, u, v), float64 arrays."""
        I = np.ascontiguousarray(I, np.int32)
        J = np.ascontiguousarray(J, np.int32)
        eta, u, v = out
        t = ctypes.c_int64()
        _chk(self.L.cliffs_gpu_get_gauges_async(self.h, len(I), _p(I, _ip), _p(J, _ip), _p(eta), _p(u), _p(v),
                                                ctypes.byref(t)), "get_gauges_async")
        return t.value

    def feed_child_async(self, nest, cuke, out):
        """Queue a feed record: out = (arrived int32 (1,), w, e (3, nn), s, n
        (3, mm)), float64; arrived[0] = 1 when the call produced a record."""
        nid, _ = nest
        a, w, e, s, n = out
        t = ctypes.c_int64()
        _chk(self.L.cliffs_gpu_feed_child_async(self.h, nid, float(cuke), _p(a, _ip), _p(w), _p(e), _p(s), _p(n),
                                                ctypes.byref(t)), "feed_child_async")
        return t.value

    def wait(self, ticket):
        _chk(self.L.cliffs_gpu_output_wait(self.h, int(ticket)), "output_wait")

    def done(self, ticket):
        d = ctypes.c_int32()
        _chk(self.L.cliffs_gpu_output_done(self.h, int(ticket), ctypes.byref(d)), "output_done")
        return bool(d.value)

    # -- profiling / tuning -------------------------------------------------------
    def profile(self, enable=True):
        _chk(self.L.cliffs_gpu_profile(self.h, int(bool(enable))), "profile")

    def profile_read(self):
        xm, ym = ctypes.c_double(), ctypes.c_double()
        xn, yn = ctypes.c_int64(), ctypes.c_int64()
        _chk(self.L.cliffs_gpu_profile_read(self.h, ctypes.byref(xm), ctypes.byref(xn),
                                            ctypes.byref(ym), ctypes.byref(yn)), "profile_read")
        return dict(x_ms=xm.value, x_n=xn.value, y_ms=ym.value, y_n=yn.value)

    def launches(self):
        """Kernels this context has launched so far."""
        n = ctypes.c_int64()
        _chk(self.L.cliffs_gpu_launch_count(self.h, ctypes.byref(n)), "launch_count")
        return int(n.value)

    def set_graph_steps(self, k):
        _chk(self.L.cliffs_gpu_set_graph_steps(self.h, int(k)), "set_graph_steps")

    def prepare_steps(self, nsteps):
        """Capture and instantiate the CUDA graphs a later step(nsteps) from
        the current state replays, without running them."""
        _chk(self.L.cliffs_gpu_prepare_steps(self.h, int(nsteps)), "prepare_steps")

    def set_tiling(self, block_x=0, warps_y=0):
        _chk(self.L.cliffs_gpu_set_tiling(self.h, int(block_x), int(warps_y)), "set_tiling")

    def set_sweep_kernel(self, kind):
        """TILED (one block per tile; the default) or STAGED (persistent, TMA-staged windows)."""
        _chk(self.L.cliffs_gpu_set_sweep_kernel(self.h, int(kind)), "set_sweep_kernel")

    def check_stage_timeout(self, wait_ms=50):
        """Failure-detection check of the staged kernels' stage waits; returns
        the library status (CLIFFS_ERR_TIMEOUT = -7 expected)."""
        return self.L.cliffs_gpu_check_stage_timeout(self.h, int(wait_ms))


class Batch:
    """Grids stepped together (cliffs_batch_*): one source scenario per grid,
    grids of any size; bit-identical to stepping each GpuGrid on its own."""

    def __init__(self, grids):
        self.L = load()
        self.grids = list(grids)
        arr = (_V * len(self.grids))(*[g.h.value if isinstance(g.h, ctypes.c_void_p) else g.h
                                       for g in self.grids])
        h = _V()
        _chk(self.L.cliffs_batch_create(arr, len(self.grids), ctypes.byref(h)), "batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.cliffs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n):
        """Advance every grid n steps; each grid's model time follows."""
        _chk(self.L.cliffs_batch_step(self.h, int(n)), "batch_step")
        for g in self.grids:
            g.t.value += n * g.dt

    def set_plan(self, mode, ctas_per_sm=1, graph_steps=32, x_rows=1, y_groups=1):
        p = BatchPlan(int(mode), int(ctas_per_sm), int(graph_steps), int(x_rows), int(y_groups))
        _chk(self.L.cliffs_batch_set_plan(self.h, ctypes.byref(p)), "batch_set_plan")

    def plan(self):
        p = BatchPlan()
        _chk(self.L.cliffs_batch_get_plan(self.h, ctypes.byref(p)), "batch_get_plan")
        return dict(mode=p.mode, ctas_per_sm=p.ctas_per_sm, graph_steps=p.graph_steps, x_rows=p.x_rows,
                    y_groups=p.y_groups)

    def autotune(self, probe_steps=8):
        ms = ctypes.c_double()
        _chk(self.L.cliffs_batch_autotune(self.h, int(probe_steps), ctypes.byref(ms)), "batch_autotune")
        return ms.value

    def set_gauges(self, gauges):
        """gauges: one (I, J) pair of 1-based index arrays per grid."""
        counts = np.array([len(I) for I, _ in gauges], np.int32)
        I = np.ascontiguousarray(np.concatenate([np.asarray(I, np.int32) for I, _ in gauges]), np.int32)
        J = np.ascontiguousarray(np.concatenate([np.asarray(J, np.int32) for _, J in gauges]), np.int32)
        _chk(self.L.cliffs_batch_set_gauges(self.h, _p(counts, _ip), _p(I, _ip), _p(J, _ip)), "batch_set_gauges")
        self.gauge_counts = counts

    def gauges(self, out=None):
        """(eta, u, v) of every grid's gauges, concatenated in grid order;
        out: three float64 arrays to fill (pinned for a fast copy)."""
        m = int(self.gauge_counts.sum())
        eta, u, v = out if out is not None else (np.empty(m), np.empty(m), np.empty(m))
        _chk(self.L.cliffs_batch_get_gauges(self.h, _p(eta), _p(u), _p(v)), "batch_get_gauges")
        return eta, u, v

    def check_barrier_timeout(self, wait_ms=100):
        """Status of a launch whose grid barrier waits for an absent block."""
        return self.L.cliffs_batch_check_barrier_timeout(self.h, int(wait_ms))

    def launches(self):
        n = ctypes.c_int64()
        _chk(self.L.cliffs_batch_launch_count(self.h, ctypes.byref(n)), "batch_launch_count")
        return int(n.value)
