"""Asynchronous outputs (cliffs_gpu_*_async): screenshots, gauge records and
child feed records queued while the steps go on, into pinned host memory,
equal to the synchronous outputs taken at the same step.

A shelf basin with a child grid near the coast steps in chunks.  At every
output point the asynchronous outputs are queued first, then the synchronous
ones are read on the same state.  More outputs are queued than the ring holds
(8), so slots are reused while earlier copies may still be in flight.  The
feed starts before the wave reaches the child: those calls report no record,
and the first record comes with the same call as the synchronous arrival."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
nested = importlib.import_module("cliffs-src_gb300.nested")
cg = pkg.cliffs_gpu
W = pkg.workloads


def test_async_outputs_equal_sync():
    c = W.shelf_2d(seed=21, nx=320, ny=256, dx=500.0, steps=0, ngauges=16, axes_km=(20, 10),
                   centre_km=(60.0, 64.0))
    g = pkg.GpuGrid.from_case(c)
    xn = np.linspace(c["xcrd"][200] + 100.0, c["xcrd"][300], 301)
    yn = np.linspace(c["ycrd"][80] + 50.0, c["ycrd"][180], 301)
    nest = g.nest_add(nested.nest_tables(c["xcrd"], c["ycrd"], xn, yn))
    mm, nn = nest[1]
    I, J = c["gauges"]
    ny, nx = c["dep"].shape
    npts = 30
    sea = [tuple(cg.pinned(((ny - 1) // 3 + 1, (nx - 1) // 2 + 1), np.float32) for _ in range(3)) for _ in range(npts)]
    gau = [tuple(cg.pinned((len(I),)) for _ in range(3)) for _ in range(npts)]
    fed = [(cg.pinned((1,), np.int32), cg.pinned((3, nn)), cg.pinned((3, nn)), cg.pinned((3, mm)),
            cg.pinned((3, mm))) for _ in range(npts)]
    tickets, sync = [], []
    arrived = False
    for k in range(npts):
        tickets.append((g.sea_state_async(2, 3, sea[k]), g.gauges_async(I, J, gau[k]),
                        g.feed_child_async(nest, 0.001, fed[k])))
        h, u, v = g.sea_state(2, 3)
        e, gu, gv = g.gauges(I, J)
        arrived, rec = g.feed_child(nest, 0.001, arrived)
        sync.append(((h, u, v), (e, gu, gv), rec))
        g.step(7)
    first = None
    for k in range(npts):
        for t in tickets[k]:
            g.wait(t)
        for a, b in zip(sea[k], sync[k][0]):
            assert np.array_equal(a, b), k
        for a, b in zip(gau[k], sync[k][1]):
            assert np.array_equal(a, b), k
        rec = sync[k][2]
        assert bool(fed[k][0][0]) == (rec is not None), k
        if rec is not None:
            first = k if first is None else first
            for a, b in zip(fed[k][1:], rec):
                assert np.array_equal(a, b), k
    assert first is not None and first > 0  # the wave reached the child during the run, not before
    g.close()
