"""Ensembles through the C ABI (cliffs_batch_*): many grids of uneven size
stepped together, by one persistent cooperative launch per call or by
per-phase launches replayed from a CUDA graph.

A batched scenario runs the same tiles with the same arithmetic as its own
sweep launches, so the checks are bit-exact against twins stepped one by one
with cliffs_gpu_step: state, max-wave fields, in both schedules, after the
autotuner (which must leave the state as it found it).  The grid barrier's
failure path is checked by its own entry point: a launch whose barrier waits
for an arrival no block makes must come back with CLIFFS_ERR_TIMEOUT after
the set limit, and the device must keep working.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
cg = pkg.cliffs_gpu
W = pkg.workloads

SIZES = [(96, 80), (160, 128), (257, 190), (64, 300), (200, 200), (129, 64)]


def _cases():
    out = []
    for k, (nx, ny) in enumerate(SIZES):
        c = W.shelf_2d(seed=50 + k, nx=nx, ny=ny, dx=400.0 + 50 * k, steps=0, amp=0.5 + 0.3 * k,
                       ngauges=0, axes_km=(20, 10), centre_km=(0.45 * nx * (400.0 + 50 * k) / 1000,
                                                            0.5 * ny * (400.0 + 50 * k) / 1000))
        c["crough"] = 0.000625 * (k % 2)
        out.append(c)
    return out


def _same(a, b):
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)


def test_batch_is_bit_identical_to_single_grids():
    cases = _cases()
    grids = [pkg.GpuGrid.from_case(c) for c in cases]
    twins = [pkg.GpuGrid.from_case(c) for c in cases]
    b = pkg.Batch(grids)
    # persistent cooperative launches
    b.set_plan(cg.PERSISTENT, ctas_per_sm=2)
    b.step(37)
    for t in twins:
        t.step(37)
    for g, t in zip(grids, twins):
        _same(g, t)
        assert abs(g.time - t.time) < 1e-9
    # per-phase launches from a graph of 8 steps (2 replays and 5 direct steps)
    b.set_plan(cg.GRAPH, graph_steps=8)
    b.step(21)
    for t in twins:
        t.step(21)
    for g, t in zip(grids, twins):
        _same(g, t)
    # tile shapes: 3 rows per x tile, 2 row groups per y tile, graphs of 8
    # steps and a tail graph of 5; then persistent with 4 x 4
    b.set_plan(cg.GRAPH, graph_steps=8, x_rows=3, y_groups=2)
    b.step(21)
    for t in twins:
        t.step(21)
    for g, t in zip(grids, twins):
        _same(g, t)
    b.set_plan(cg.PERSISTENT, ctas_per_sm=1, x_rows=4, y_groups=4)
    b.step(9)
    for t in twins:
        t.step(9)
    for g, t in zip(grids, twins):
        _same(g, t)
    # the autotuner probes every plan from a snapshot and restores it
    before = [g.download_state() for g in grids]
    ms = b.autotune(4)
    assert ms > 0
    plan = b.plan()
    assert plan["mode"] in (cg.PERSISTENT, cg.GRAPH)
    assert plan["x_rows"] in (1, 2, 4) and plan["y_groups"] in (1, 2, 4)
    for g, st in zip(grids, before):
        for x, y in zip(g.download_state(), st):
            assert np.array_equal(x, y)
    b.step(10)
    for t in twins:
        t.step(10)
    for g, t in zip(grids, twins):
        _same(g, t)
        assert g.status() == (0, 0)
    assert b.launches() > 0
    b.close()


def test_batch_barrier_timeout_is_reported():
    cases = _cases()[:2]
    grids = [pkg.GpuGrid.from_case(c) for c in cases]
    b = pkg.Batch(grids)
    assert b.check_barrier_timeout(100) == cg.CliffsError(-7, "x").code
    # the device and the batch keep working
    for g, c in zip(grids, cases):
        g.set_initial(c["H0"], c.get("u0"), c.get("v0"))
    b.set_plan(cg.PERSISTENT, ctas_per_sm=1)
    b.step(5)
    twins = [pkg.GpuGrid.from_case(c) for c in cases]
    for t in twins:
        t.step(5)
    for g, t in zip(grids, twins):
        for x, y in zip(g.download_state(), t.download_state()):
            assert np.array_equal(x, y)
    b.close()


def test_batch_rejects_what_it_cannot_step():
    c2 = _cases()[0]
    c1 = W.channel_1d(seed=1, n=300, steps=0)
    g2 = pkg.GpuGrid.from_case(c2)
    g1 = pkg.GpuGrid.from_case(c1)
    with pytest.raises(cg.CliffsError):
        pkg.Batch([g2, g1])  # a 1-D grid
    nt = 4
    g2.set_feed(np.arange(nt) * 10.0, np.zeros((nt, 3, c2["dep"].shape[0])),
                np.zeros((nt, 3, c2["dep"].shape[0])), np.zeros((nt, 3, c2["dep"].shape[1])),
                np.zeros((nt, 3, c2["dep"].shape[1])), irec=2, freeze=False)
    with pytest.raises(cg.CliffsError):
        pkg.Batch([g2])  # boundary forcing is per grid


def test_batch_with_rising_sources_is_bit_identical():
    cases = _cases()[:4]
    grids = [pkg.GpuGrid.from_case(c) for c in cases]
    twins = [pkg.GpuGrid.from_case(c) for c in cases]
    for k, (g, t, c) in enumerate(zip(grids, twins, cases)):
        L = c["xcrd"][-1]
        src = dict(x0=0.4 * L, y0=0.5 * c["ycrd"][-1], ax=0.15 * L, ay=0.1 * L, angle=0.3 * k, amp=1.0,
                   dipole=0.2, rise_time=(3 + 4 * k) * c["dt"] if k % 2 == 0 else 0.0)
        g.add_source(c["xcrd"], c["ycrd"], **src)
        t.add_source(c["xcrd"], c["ycrd"], **src)
    b = pkg.Batch(grids)
    b.set_plan(cg.GRAPH, graph_steps=8)
    b.step(30)
    for t in twins:
        t.step(30)
    for g, t in zip(grids, twins):
        _same(g, t)
    b.close()


def test_batch_after_single_steps_and_reads():
    """Contexts that stepped alone join a batch with their last end state
    pending; the batch's x-sweeps fold it in.  Reads of the max-wave fields
    between batched steps, and single steps after them, keep the fields equal
    to those of twins that never joined a batch."""
    cases = _cases()[:3]
    grids = [pkg.GpuGrid.from_case(c) for c in cases]
    twins = [pkg.GpuGrid.from_case(c) for c in cases]
    for g in grids + twins:
        g.step(7)
    b = pkg.Batch(grids)
    for plan in ((cg.PERSISTENT, dict(ctas_per_sm=1)), (cg.GRAPH, dict(graph_steps=8))):
        b.set_plan(plan[0], **plan[1])
        b.step(20)
        for t in twins:
            t.step(20)
        for g, t in zip(grids, twins):
            _same(g, t)
    for g in grids + twins:
        g.step(3)
    for g, t in zip(grids, twins):
        _same(g, t)
    b.close()


def test_batch_gauges_match_single_grids():
    """cliffs_batch_get_gauges samples every scenario's gauges in one launch;
    the records equal each twin's own cliffs_gpu_get_gauges bit for bit,
    at the start and after batched steps."""
    cases = _cases()
    rng = np.random.default_rng(5)
    gauges = []
    for c in cases:
        ny, nx = c["dep"].shape
        m = int(rng.integers(1, 9))
        gauges.append((rng.integers(1, nx + 1, m).astype(np.int32), rng.integers(1, ny + 1, m).astype(np.int32)))
    grids = [pkg.GpuGrid.from_case(c) for c in cases]
    twins = [pkg.GpuGrid.from_case(c) for c in cases]
    b = pkg.Batch(grids)
    b.set_gauges(gauges)
    b.set_plan(cg.GRAPH, graph_steps=8, x_rows=2, y_groups=2)
    for n in (0, 13, 8):
        if n:
            b.step(n)
            for t in twins:
                t.step(n)
        eta, u, v = b.gauges()
        k = 0
        for t, (I, J) in zip(twins, gauges):
            te, tu, tv = t.gauges(I, J)
            m = len(I)
            assert np.array_equal(eta[k:k + m], te) and np.array_equal(u[k:k + m], tu)
            assert np.array_equal(v[k:k + m], tv)
            k += m
    b.close()
