"""Plain steps replayed from a CUDA graph (cliffs_gpu_set_graph_steps) are
bit-identical to launching every sweep, including a step count that is not a
multiple of the graph's length and a single sweep in between (which changes
the state copy the graph was captured with)."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads


def test_graph_steps_bit_identical():
    c = W.shelf_2d(seed=81, nx=300, ny=220, dx=500.0, steps=0, ngauges=0, axes_km=(30, 15),
                   centre_km=(60.0, 55.0))
    c["crough"] = 0.000625
    a = pkg.GpuGrid.from_case(c)
    b = pkg.GpuGrid.from_case(c)
    b.set_graph_steps(0)
    for n in (37, 16, 5):
        a.step(n)
        b.step(n)
    a.sweep(1)  # one x-sweep: the other state copy is now current
    b.sweep(1)
    a.step(40)
    b.step(40)
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)
    assert a.launches() == b.launches()
    assert abs(a.time - b.time) < 1e-9
    a.close()
    b.close()
