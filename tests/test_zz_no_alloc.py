"""The sweep entry point that allocates no device memory.

cliffs_gpu_sweep_noalloc serves callers that cannot allocate device memory:
applications that give the solver a fixed memory budget and forbid cudaMalloc
afterwards, or time loops that cannot afford cudaMalloc's implicit device
synchronisation.  Its scratch (the worklist of shoreline cells) is a fixed
array compiled into the library.  These tests call it through the C ABI on
device buffers the test owns, and check two calls in a row (an x-sweep, then a
y-sweep on its output) against the same sweeps through the regular,
allocating context API.  Collected last on purpose: the file name sorts after
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


def test_noalloc_matches_context_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = pkg.load()
    case = pkg.workloads.shelf_2d(seed=7, nx=300, ny=260, dx=800.0, steps=0, ngauges=0)
    case["crough"] = 0.000625
    ny, nx = case["dep"].shape
    dx = float(case["xcrd"][1] - case["xcrd"][0])
    dy = float(case["ycrd"][1] - case["ycrd"][0])
    # regular context: advance a few steps so that the state is not trivial
    g = pkg.GpuGrid.from_case(case)
    g.step(40)
    cel, u, v = g.download_state()
    dep = case["dep"]
    pitch = (nx + 31) // 32 * 32
    d_dep = _dev(torch, dep, pitch)
    bufs = [[_dev(torch, a, pitch) for a in (_to_surface_state(cel, dep), u, v)],
            [torch.zeros((ny, pitch), dtype=torch.float32, device="cuda") for _ in range(3)]]
    stream = torch.cuda.current_stream().cuda_stream
    src = 0
    for call, iu in enumerate((1, 2)):
        a, b = bufs[src], bufs[1 - src]
        r = L.cliffs_gpu_sweep_noalloc(iu, nx, ny, pitch, d_dep.data_ptr(), a[0].data_ptr(),
                                       a[1].data_ptr(), a[2].data_ptr(), b[0].data_ptr(),
                                       b[1].data_ptr(), b[2].data_ptr(), dx, dy, case["ground"],
                                       case["crough"], case["dt"], ctypes.c_void_p(stream))
        assert r == 0, (call, r)
        torch.cuda.synchronize()
        g.sweep(iu)  # the same sweep through the allocating API
        cg, ug, vg = g.download_state()
        srf_ref = _to_surface_state(cg, dep)
        srf_na = b[0][:, :nx].cpu().numpy().astype(np.float64)
        # same kernels, same arithmetic: agreement well inside the parity
        # tolerance of the suite (1e-4 of a 2 m source amplitude)
        assert np.abs(srf_na - srf_ref).max() <= 1e-6, call
        assert np.abs(b[1][:, :nx].cpu().numpy() - ug).max() <= 1e-7, call
        assert np.abs(b[2][:, :nx].cpu().numpy() - vg).max() <= 1e-7, call
        src = 1 - src
    g.close()


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
