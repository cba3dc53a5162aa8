"""Transfers with the caller's arrays in pinned host memory.

When the host arrays of cliffs_gpu_set_initial / upload_state,
cliffs_gpu_download_state and cliffs_gpu_get_maxwave are pinned
(cliffs_gpu_host_alloc), the conversion kernels read and write them in place
instead of going through the device staging area and the copy engines.  The
results must be the same bits as with pageable arrays: the same initial
state, the same steps, the same downloads and max-wave fields.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads
cg = pkg.cliffs_gpu


def _case():
    c = W.shelf_2d(seed=33, nx=300, ny=220, dx=500.0, steps=0, ngauges=0, axes_km=(30, 15),
                   centre_km=(120.0, 55.0))
    c["crough"] = 0.000625
    c["u0"] = 0.01 * np.sin(np.arange(c["dep"].size)).reshape(c["dep"].shape)
    c["v0"] = 0.01 * np.cos(np.arange(c["dep"].size)).reshape(c["dep"].shape)
    return c


def _pin(a, dtype=np.float64):
    p = cg.pinned(a.shape, dtype)
    p[...] = a
    return p


def test_pinned_transfers_equal_pageable():
    c = _case()
    a = pkg.GpuGrid.from_case(c)  # pageable initial state
    dx, rs, dy, zeta = cg.metrics(c["xcrd"], c["ycrd"], c["cartesian"])
    b = pkg.GpuGrid(_pin(c["dep"]), dx=dx, row_scale=rs, dy=dy, zeta=zeta, ground=c["ground"], crough=c["crough"],
                    dt=c["dt"])
    b.set_initial(_pin(c["H0"]), _pin(c["u0"]), _pin(c["v0"]))  # read in place
    ny, nx = c["dep"].shape
    for steps in (0, 120):
        if steps:
            a.step(steps)
            b.step(steps)
        ref = a.download_state()
        got = b.download_state(out=[cg.pinned((ny, nx)) for _ in range(3)])  # written in place
        for x, y in zip(ref, got):
            assert np.array_equal(x, y)
        mref = a.maxwave()
        mgot = b.maxwave(out=[cg.pinned((ny, nx), np.float32) for _ in range(2)])
        for x, y in zip(mref, mgot):
            assert np.array_equal(x, y, equal_nan=True)
    # a download of the celerity alone into a pinned array (the others not asked for)
    cel = cg.pinned((ny, nx))
    r = b.L.cliffs_gpu_download_state(b.h, cg._p(cel), None, None)
    assert r == 0 and np.array_equal(cel, ref[0])
    # upload_state from pinned arrays, then the same steps on both
    a.upload_state(*ref)
    b.upload_state(*[_pin(x) for x in ref])
    a.step(30)
    b.step(30)
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    assert a.status()[0] == 0 and b.status()[0] == 0
    a.close()
    b.close()
