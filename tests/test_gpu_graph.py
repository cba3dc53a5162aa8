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


def test_tail_graphs_and_prepared_graphs_bit_identical():
    """The last steps of a call (fewer than graph_k) replay from a graph of
    their own length; prepare_steps instantiates the graphs before the call.
    Both are bit-identical to a launch per sweep."""
    c = W.shelf_2d(seed=82, nx=260, ny=200, dx=500.0, steps=0, ngauges=0, axes_km=(30, 15),
                   centre_km=(55.0, 50.0))
    c["crough"] = 0.000625
    a = pkg.GpuGrid.from_case(c)
    b = pkg.GpuGrid.from_case(c)
    b.set_graph_steps(0)
    a.set_graph_steps(16)
    a.prepare_steps(21)  # fresh state: 1 step alone, then graphs of 16 and 4
    for n in (21, 4, 7, 3, 2, 16, 9, 7):  # tails 4, 7, 3, 2, 9: more lengths than the cache keeps
        a.step(n)
        b.step(n)
    a.prepare_steps(20)
    a.step(20)
    b.step(20)
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)
    assert a.launches() == b.launches()
    assert abs(a.time - b.time) < 1e-9
    a.close()
    b.close()


@pytest.mark.parametrize("k", [16, 7])
def test_one_dimensional_graphs_keep_the_state_copy(k):
    """A 1-D grid sweeps once per step: graphs take an even number of steps,
    so an odd graph_k or an odd tail still ends on the state copy it began
    from.  Bit-identical to a launch per sweep."""
    c = W.channel_1d(seed=13, n=2000, dx=0.05, steps=0)
    a = pkg.GpuGrid.from_case(c)
    b = pkg.GpuGrid.from_case(c)
    b.set_graph_steps(0)
    a.set_graph_steps(k)
    for n in (1, 23, 16, 5, 300, 3, 1, 64):
        a.step(n)
        b.step(n)
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)
    assert a.launches() == b.launches()
    a.close()
    b.close()
