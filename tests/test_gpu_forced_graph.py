"""Forced steps replayed from CUDA graphs (a ring of per-step edge tables
filled by one kernel per chunk) are bit-identical to a launch per sweep with
the forcing interpolated per step: states, max-wave fields, model time, the
record cursor's stop with and without freeze, and calls of every length
around the graph's (cliffs_main.f:305-339)."""
import importlib

import numpy as np
import pytest

from test_gpu_features import _records

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads


def _forced_pair(freeze, k):
    case = W.shelf_2d(seed=21, nx=160, ny=120, dx=1000.0, steps=0, amp=0.0, ngauges=8, perturb=0.02)
    ny, nx = case["dep"].shape
    nt = 30
    tin = np.arange(nt) * 8 * case["dt"]
    recs = (_records(nt, ny, tin, 0.4, 0.0), _records(nt, ny, tin, 0.1, 0.3), _records(nt, nx, tin, 0.2, 0.1),
            _records(nt, nx, tin, 0.05, 0.6))
    grids = []
    for graph_k in (k, 0):  # graphs of k steps, and a launch per sweep
        g = pkg.GpuGrid.from_case(case)
        g.set_graph_steps(graph_k)
        g.set_feed(tin, *recs, irec=2, freeze=freeze)
        g.t.value = tin[1]
        grids.append(g)
    return grids, tin, case["dt"]


@pytest.mark.parametrize("freeze,k", [(True, 16), (False, 16), (False, 5)])
def test_forced_graph_steps_bit_identical(freeze, k):
    (a, b), tin, dt = _forced_pair(freeze, k)
    total = int((tin[-1] - tin[1]) / dt) + 40  # past the last record
    done = 0
    for n in (1, 3 * k, k - 1, 2 * k + 7, total):
        ra, rb = a.step(n), b.step(n)
        assert ra == rb
        assert a.time == b.time
        for x, y in zip(a.download_state(), b.download_state()):
            assert np.array_equal(x, y)
        done += ra[0]
        if ra[1]:  # the forcing ended with freeze
            break
    assert (done < 1 + 3 * k + k - 1 + 2 * k + 7 + total) == freeze
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)
    assert a.status()[0] == 0 and b.status()[0] == 0
    assert a.launches() < b.launches()  # the graphs ran
    a.close()
    b.close()
