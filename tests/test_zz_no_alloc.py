"""The sweep entry point that allocates no device memory.

cliffs_gpu_sweep_noalloc serves callers that cannot allocate device memory:
applications that give the solver a fixed memory budget and forbid cudaMalloc
afterwards, or time loops that cannot afford cudaMalloc's implicit device
synchronisation.  Its scratch (the worklist of shoreline cells) is a fixed
array compiled into the library.  These tests call it through the C ABI on
device buffers the test owns, and check two calls in a row (an x-sweep, then a
y-sweep on its output; two x-sweeps on a 1-D row; a grid at exactly the
2^20-cell limit) against the same sweeps through the regular, allocating
context API, and that a non-finite result is reported by the status reader.  Collected last on purpose: the file name sorts after
every other test module.
"""
import ctypes
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
GRAV = 9.800000190734863


def _to_surface_state(cel, dep):
    """Celerity form (the context's download) -> the library's surface state:
    eta where dep >= 0, the water depth H where dep < 0 (on FP32 depths)."""
    d = dep.astype(np.float32).astype(np.float64)
    H = cel * np.abs(cel) / GRAV
    return np.where(d < 0, H, H - d)


def _dev(torch, a2d, pitch):
    ny, nx = a2d.shape
    t = torch.zeros((ny, pitch), dtype=torch.float32, device="cuda")
    t[:, :nx] = torch.from_numpy(np.ascontiguousarray(a2d, np.float32)).cuda()
    return t


def _status(L, stream):
    flags, listed = ctypes.c_uint32(0), ctypes.c_uint32(0)
    r = L.cliffs_gpu_sweep_noalloc_status(ctypes.c_void_p(stream), ctypes.byref(flags), ctypes.byref(listed))
    return r, flags.value, listed.value


def _run_against_context(torch, case, warm_steps, sweeps, pitch=None):
    """Advance a context warm_steps steps, then apply `sweeps` (a sequence of
    iu) both through cliffs_gpu_sweep_noalloc, each call reading the previous
    call's output, and through the context's own sweeps.  Returns the cells
    each no-alloc call listed for the full wet/dry rules."""
    L = pkg.load()
    ny, nx = case["dep"].shape
    dx = float(case["xcrd"][1] - case["xcrd"][0]) if nx > 1 else 1.0
    dy = float(case["ycrd"][1] - case["ycrd"][0]) if ny > 1 else 1.0
    g = pkg.GpuGrid.from_case(case)
    if warm_steps:
        g.step(warm_steps)
    cel, u, v = g.download_state()
    dep = case["dep"]
    pitch = pitch or (nx + 31) // 32 * 32
    d_dep = _dev(torch, dep, pitch)
    bufs = [[_dev(torch, a, pitch) for a in (_to_surface_state(cel, dep), u, v)],
            [torch.zeros((ny, pitch), dtype=torch.float32, device="cuda") for _ in range(3)]]
    stream = torch.cuda.current_stream().cuda_stream
    src = 0
    listed = []
    for call, iu in enumerate(sweeps):
        a, b = bufs[src], bufs[1 - src]
        r = L.cliffs_gpu_sweep_noalloc(iu, nx, ny, pitch, d_dep.data_ptr(), a[0].data_ptr(),
                                       a[1].data_ptr(), a[2].data_ptr(), b[0].data_ptr(),
                                       b[1].data_ptr(), b[2].data_ptr(), dx, dy, case["ground"],
                                       case["crough"], case["dt"], ctypes.c_void_p(stream))
        assert r == 0, (call, r)
        rs, flags, n = _status(L, stream)
        assert rs == 0 and flags == 0, (call, rs, flags)
        listed.append(n)
        g.sweep(iu)  # the same sweep through the allocating API
        cg, ug, vg = g.download_state()
        srf_ref = _to_surface_state(cg, dep)
        srf_na = b[0][:, :nx].cpu().numpy().astype(np.float64)
        # same kernels, same arithmetic: agreement well inside the parity
        # tolerance of the suite (1e-4 of the source amplitude)
        assert np.abs(srf_na - srf_ref).max() <= 1e-6, call
        assert np.abs(b[1][:, :nx].cpu().numpy() - ug).max() <= 1e-7, call
        assert np.abs(b[2][:, :nx].cpu().numpy() - vg).max() <= 1e-7, call
        src = 1 - src
    g.close()
    return listed


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def test_noalloc_matches_context_two_calls():
    torch = _torch()
    case = pkg.workloads.shelf_2d(seed=7, nx=300, ny=260, dx=800.0, steps=0, ngauges=0)
    case["crough"] = 0.000625
    listed = _run_against_context(torch, case, 40, (1, 2))
    # the shelf's coast crosses every row: the x-sweep took cells through the
    # worklist kernel (general_kernel), not the fast path alone
    assert listed[0] > 0, listed


def test_noalloc_one_dimensional_row():
    """A 1-D grid (ny = 1): the x-sweep runs row 1 only.  After 1500 steps the
    solitary wave is on the beach, so the shoreline cells take the worklist."""
    torch = _torch()
    case = pkg.workloads.channel_1d(seed=13, n=2000, dx=0.05, steps=0)
    listed = _run_against_context(torch, case, 1500, (1, 1))
    assert min(listed) > 0, listed


def test_noalloc_at_the_size_limit():
    """Exactly 1024 x 1024 = 2^20 cells, the largest grid the fixed scratch
    takes, with pitch = nx."""
    torch = _torch()
    case = pkg.workloads.shelf_2d(seed=5, nx=1024, ny=1024, dx=200.0, steps=0, ngauges=0)
    listed = _run_against_context(torch, case, 20, (1, 2), pitch=1024)
    assert listed[0] > 0, listed


def test_noalloc_reports_non_finite_and_clears_it():
    """A non-finite input value sets CLIFFS_ST_NAN, which the status reader
    returns as CLIFFS_ERR_NAN; the next clean call starts from a cleared word."""
    torch = _torch()
    L = pkg.load()
    case = pkg.workloads.shelf_2d(seed=7, nx=300, ny=260, dx=800.0, steps=0, ngauges=0)
    ny, nx = case["dep"].shape
    dx = float(case["xcrd"][1] - case["xcrd"][0])
    pitch = (nx + 31) // 32 * 32
    d_dep = _dev(torch, case["dep"], pitch)
    # the initial state as cliffs_gpu_set_initial forms it: H = 0 where the
    # total depth is at most ground (cliffs_main.f:218-227)
    H = np.where(case["H0"] <= case["ground"], 0.0, case["H0"])
    d32 = case["dep"].astype(np.float32).astype(np.float64)
    state = [_dev(torch, a, pitch) for a in (np.where(d32 < 0, H, H - case["dep"]), case["u0"], case["v0"])]
    out = [torch.zeros((ny, pitch), dtype=torch.float32, device="cuda") for _ in range(3)]
    stream = torch.cuda.current_stream().cuda_stream
    wet = np.argwhere(case["dep"] > 100.0)[len(np.argwhere(case["dep"] > 100.0)) // 2]

    def call():
        return L.cliffs_gpu_sweep_noalloc(1, nx, ny, pitch, d_dep.data_ptr(), state[0].data_ptr(),
                                          state[1].data_ptr(), state[2].data_ptr(), out[0].data_ptr(),
                                          out[1].data_ptr(), out[2].data_ptr(), dx, dx, case["ground"],
                                          case["crough"], case["dt"], ctypes.c_void_p(stream))

    keep = float(state[0][wet[0], wet[1]])
    state[0][wet[0], wet[1]] = float("nan")
    assert call() == 0
    r, flags, _ = _status(L, stream)
    assert r == -3 and flags & 1, (r, flags)
    state[0][wet[0], wet[1]] = keep
    assert call() == 0
    r, flags, _ = _status(L, stream)
    assert r == 0 and flags == 0, (r, flags)


def test_noalloc_rejects_oversized_and_misaligned():
    L = pkg.load()
    null = ctypes.c_void_p(16)  # never dereferenced: the checks come first
    args = [null] * 7
    # beyond the fixed scratch: 2048 x 1024 cells > 2^20
    assert L.cliffs_gpu_sweep_noalloc(1, 2048, 1024, 2048, *args, 1.0, 1.0, 0.01, 0.0, 0.1, None) == -1
    # pitch not a multiple of 4
    assert L.cliffs_gpu_sweep_noalloc(1, 100, 100, 101, *args, 1.0, 1.0, 0.01, 0.0, 0.1, None) == -1
    # a sweep direction the grid shape does not run
    assert L.cliffs_gpu_sweep_noalloc(2, 100, 2, 100, *args, 1.0, 1.0, 0.01, 0.0, 0.1, None) == -1
