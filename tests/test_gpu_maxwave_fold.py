"""Max-wave bookkeeping of two-dimensional steps with the tiled kernels: the
x-sweep folds the previous step's end state into hmax/velmax (cliffs_main.f:
347-355 moved one sweep later), and max_sync folds the latest one in before
any read or any change of the state outside a step.  The staged kernels still
update the fields in the y-sweep, with the step's own outputs; both kernel
sets give bit-identical states, so their max-wave fields must agree after
every kind of call that touches them:

  the first step from the initial state (nothing folded in), reads in the
  middle of a run, graph replays after a read, single sweeps, a state
  uploaded in mid-run, an instantaneous and a rising source, the runup
  measure, an explicit maxwave_update, and a switch of kernels in mid-run."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pkg = importlib.import_module("cliffs-src_gb300")
W = pkg.workloads
cg = pkg.cliffs_gpu


def _case():
    c = W.shelf_2d(seed=81, nx=300, ny=220, dx=500.0, steps=0, ngauges=0, axes_km=(30, 15),
                   centre_km=(120.0, 55.0))
    c["crough"] = 0.000625
    return c


def _pair():
    c = _case()
    a = pkg.GpuGrid.from_case(c)  # tiled: the fold
    b = pkg.GpuGrid.from_case(c)
    b.set_sweep_kernel(cg.STAGED)  # the update in the y-sweep
    return c, a, b


def _same_max(a, b):
    for x, y in zip(a.maxwave(), b.maxwave()):
        assert np.array_equal(x, y)
    for x, y in zip(a.max_raw(), b.max_raw()):
        assert np.array_equal(x, y)


def test_fold_equals_update_in_the_y_sweep():
    c, a, b = _pair()
    src = dict(x0=float(c["xcrd"][150]), y0=float(c["ycrd"][110]), ax=8e3, ay=5e3, amp=0.3)
    calls = [
        lambda g: g.step(1),                # the first step: the initial state is not folded in
        None,
        lambda g: g.step(40),               # a graph replay after a read
        None,
        lambda g: g.sweep(1),               # a half step by hand
        lambda g: g.sweep(2),
        lambda g: g.maxwave_update(),       # the caller's own update after it
        lambda g: g.step(17),
        None,
        lambda g: g.upload_state(*g.download_state()),
        lambda g: g.step(5),
        lambda g: g.add_source(c["xcrd"], c["ycrd"], **src),
        lambda g: g.step(16),
        lambda g: g.runup(),
        lambda g: g.add_source(c["xcrd"], c["ycrd"], **src, rise_time=4 * c["dt"]),
        lambda g: g.step(21),
        None,
        lambda g: g.step(9),
        lambda g: g.set_sweep_kernel(cg.STAGED),  # a pending end state, then the other kernels
        lambda g: g.step(12),
        lambda g: g.set_sweep_kernel(cg.TILED),
        lambda g: g.step(12),
        None,
    ]
    for f in calls:
        if f is None:
            _same_max(a, b)
            continue
        assert f(a) == f(b)
    for x, y in zip(a.download_state(), b.download_state()):
        assert np.array_equal(x, y)
    _same_max(a, b)
    # the caller's own output arrays are filled in place
    st = [np.full((a.ny, a.nx), 7.0) for _ in range(3)]
    mw = [np.full((a.ny, a.nx), 7.0, np.float32) for _ in range(2)]
    assert all(x is y for x, y in zip(a.download_state(out=st), st))
    assert all(x is y for x, y in zip(a.maxwave(out=mw), mw))
    for x, y in zip(st, b.download_state()):
        assert np.array_equal(x, y)
    for x, y in zip(mw, b.maxwave()):
        assert np.array_equal(x, y)
    with pytest.raises(ValueError):
        a.maxwave(out=[np.zeros((a.ny, a.nx))] * 2)  # float64 where float32 is due
    assert a.status()[0] == 0 and b.status()[0] == 0
    a.close()
    b.close()


def test_first_step_leaves_the_initial_state_out():
    """The max-wave fields start at zero (cliffs_main.f:196-197) and take the
    end state of every step, never the initial state: after one step MaxE is
    that step's surface, also where the initial uplift has already fallen."""
    c = _case()
    X, Y = np.meshgrid(c["xcrd"], c["ycrd"])
    hump = 2.0 * np.exp(-((X - c["xcrd"][100]) ** 2 + (Y - c["ycrd"][110]) ** 2) / 3e3 ** 2)
    c["H0"] = np.where(c["dep"] > 0, c["H0"] + hump, c["H0"])  # a sharp hump at sea, falling from the start
    a = pkg.GpuGrid.from_case(c)
    b = pkg.GpuGrid.from_case(c)
    b.set_sweep_kernel(cg.STAGED)
    eta0 = a.eta()
    a.step(1)
    b.step(1)
    eta1 = a.eta()
    me, _ = a.maxwave()
    wet = np.isfinite(eta1) & np.isfinite(eta0)
    assert (eta1[wet] < eta0[wet] - 2e-3).any()  # the case tells the two apart
    assert np.abs(me[wet] - eta1[wet]).max() < 1e-4
    _same_max(a, b)
    a.close()
    b.close()
