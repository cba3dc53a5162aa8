"""The oracle's restatement of ComputeBoundaryInput (cmpboundary/scan4wave.f,
get_sea_state.f, InterpolateOntoBndr.f), pinned on the CPU by hand-worked
cases and by a second, vectorised restatement in numpy:

- scan4wave.f: the first record whose largest value or largest negated value
  is above cuke, values below -1e10 counting as 0; nt + 1 when none is (the
  DO loop's index after it ran out).  The reference reports any result >= nt
  as "no signal above treshold".
- get_sea_state.f: with units other than m the values are times 0.01 as a
  real*4 product, before the FP64 interpolation.
- InterpolateOntoBndr.f:6-38: across the edge first (between the lattice
  columns or rows that straddle it), then along it; a linear field comes back
  at the edge nodes.
"""
import numpy as np
import pytest

import oracle


def _tables(x, y, xn, yn):
    return oracle.NestTables(x, y, xn, yn)


def _footprint(t, field):
    """The footprint of the target in a (nt, NY, NX) cube, as the tool cuts
    it: columns W_nx .. E_nx+1, rows S_ny .. N_ny+1 (1-based)."""
    d = t.as_dict()
    return np.ascontiguousarray(field[:, d["S_ny"] - 1:d["N_ny"] + 1, d["W_nx"] - 1:d["E_nx"] + 1])


def _edges_numpy(t, cube, ival, scale, out):
    """InterpolateOntoBndr.f restated with numpy arrays, one rounding per
    operation as the reference's expressions: column/row first, then along
    the edge."""
    d = t.as_dict()
    sea = cube.astype(np.float32).copy()
    sea[sea < -1.0e10] = 0.0
    if scale != 1.0:
        sea = sea * np.float32(scale)
    sea = sea.astype(np.float64)                      # (nt, ny, nx)
    w, e, s, n = out
    wc = d["W_cx"] * sea[:, :, 0] + (1 - d["W_cx"]) * sea[:, :, 1]
    ec = d["E_cx"] * sea[:, :, -2] + (1 - d["E_cx"]) * sea[:, :, -1]
    kk = d["WE_ny"] - d["WE_ny"][0]
    cc = d["WE_cy"]
    w[:, ival - 1, :] = cc * wc[:, kk] + (1 - cc) * wc[:, kk + 1]
    e[:, ival - 1, :] = cc * ec[:, kk] + (1 - cc) * ec[:, kk + 1]
    sr = d["S_cy"] * sea[:, 0, :] + (1 - d["S_cy"]) * sea[:, 1, :]
    nr = d["N_cy"] * sea[:, -2, :] + (1 - d["N_cy"]) * sea[:, -1, :]
    kk = d["SN_nx"] - d["SN_nx"][0]
    cc = d["SN_cx"]
    s[:, ival - 1, :] = cc * sr[:, kk] + (1 - cc) * sr[:, kk + 1]
    n[:, ival - 1, :] = cc * nr[:, kk] + (1 - cc) * nr[:, kk + 1]


def test_scan_first_record():
    c = np.zeros((6, 4, 5), np.float32)
    c[3, 2, 1] = 0.5
    assert oracle.boundary_scan(c, 0.1) == 4
    c[1, 0, 4] = -0.25                                  # a trough counts as well
    assert oracle.boundary_scan(c, 0.1) == 2


def test_scan_threshold_is_strict():
    c = np.zeros((4, 3, 3), np.float32)
    c[1, 1, 1] = 0.5
    assert oracle.boundary_scan(c, 0.5) == 5            # equal to cuke is still sea
    assert oracle.boundary_scan(c, np.nextafter(0.5, 0.0)) == 2


def test_scan_missing_values_are_still_sea():
    c = np.full((5, 3, 4), -1.0e20, np.float32)        # missing: below -1e10
    assert oracle.boundary_scan(c, 0.1) == 6
    c[2, 0, 0] = -1.0e10                               # exactly -1e10 is a value, and deep
    assert oracle.boundary_scan(c, 0.1) == 3


def test_scan_last_record_and_none():
    """A first signal at the last record gives nt, none gives nt + 1: both
    are 'no signal' to the reference (it >= nt)."""
    c = np.zeros((7, 2, 2), np.float32)
    assert oracle.boundary_scan(c, 0.01) == 8
    c[6, 1, 1] = 1.0
    assert oracle.boundary_scan(c, 0.01) == 7
    c[5, 0, 0] = 1.0
    assert oracle.boundary_scan(c, 0.01) == 6


def test_edges_hand_worked():
    """Lattice x 0..3, y 0..2; target x 0.5..1.5, y 0.25..1.75; the field
    v = 10 (x + 1) + (y + 1) at every record.  The weights are dyadic, so
    the edge values are the field's values at the edge nodes exactly."""
    x, y = np.arange(4.0), np.arange(3.0)
    xn, yn = np.array([0.5, 1.0, 1.5]), np.array([0.25, 1.0, 1.75])
    t = _tables(x, y, xn, yn)
    d = t.as_dict()
    assert (d["W_nx"], d["E_nx"], d["S_ny"], d["N_ny"]) == (1, 2, 1, 2)
    assert (d["W_cx"], d["E_cx"], d["S_cy"], d["N_cy"]) == (0.5, 0.5, 0.75, 0.25)
    field = (10 * (x[None, :] + 1) + (y[:, None] + 1))[None].repeat(2, 0).astype(np.float32)
    cube = _footprint(t, field)
    assert cube.shape == (2, 3, 3)
    w, e, s, n = oracle.boundary_edges(t, [cube, 2 * cube, 3 * cube])
    for ival in (1, 2, 3):
        np.testing.assert_array_equal(w[:, ival - 1], ival * (10 * 1.5 + yn + 1)[None].repeat(2, 0))
        np.testing.assert_array_equal(e[:, ival - 1], ival * (10 * 2.5 + yn + 1)[None].repeat(2, 0))
        np.testing.assert_array_equal(s[:, ival - 1], ival * (10 * (xn + 1) + 1.25)[None].repeat(2, 0))
        np.testing.assert_array_equal(n[:, ival - 1], ival * (10 * (xn + 1) + 2.75)[None].repeat(2, 0))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_edges_reproduce_a_linear_field(seed):
    rng = np.random.default_rng(seed)
    x = np.cumsum(rng.uniform(0.5, 1.5, 40))
    y = np.cumsum(rng.uniform(0.5, 1.5, 30))
    xn = np.linspace(rng.uniform(x[2], x[8]), rng.uniform(x[25], x[-1]), 57)
    yn = np.linspace(rng.uniform(y[0], y[5]), rng.uniform(y[20], y[-1]), 43)
    t = _tables(x, y, xn, yn)
    a, b, c = rng.uniform(-1, 1, 3)
    field = (a + b * x[None, :] + c * y[:, None])[None].astype(np.float32)
    w, e, s, n = oracle.boundary_edges(t, [_footprint(t, field)] * 3)
    tol = 1e-5 * (1 + abs(b) * x[-1] + abs(c) * y[-1])
    np.testing.assert_allclose(w[0, 2], a + b * xn[0] + c * yn, atol=tol)
    np.testing.assert_allclose(e[0, 2], a + b * xn[-1] + c * yn, atol=tol)
    np.testing.assert_allclose(s[0, 2], a + b * xn + c * yn[0], atol=tol)
    np.testing.assert_allclose(n[0, 2], a + b * xn + c * yn[-1], atol=tol)


@pytest.mark.parametrize("scale", [1.0, 0.01])
def test_edges_match_numpy_restatement(scale):
    rng = np.random.default_rng(7)
    x = np.linspace(130.0, 150.0, 61)
    y = np.linspace(30.0, 45.0, 46)
    xn = np.linspace(137.13, 141.71, 211)
    yn = np.linspace(35.02, 38.93, 187)
    t = _tables(x, y, xn, yn)
    field = rng.normal(0.0, 50.0, (3, 9, 46, 61)).astype(np.float32)
    field[rng.random(field.shape) < 0.05] = -1.0e30     # missing values
    cubes = [_footprint(t, f) for f in field]
    got = oracle.boundary_edges(t, cubes, scale)
    ref = tuple(np.zeros_like(g) for g in got)
    for ival, cube in enumerate(cubes, start=1):
        _edges_numpy(t, cube, ival, scale, ref)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


def test_centimetres_scale_is_single_precision():
    """get_sea_state.f: sea = 0.01*sea on real*4 values, a real*4 product;
    the interpolation then runs in FP64 on the product."""
    x, y = np.arange(3.0), np.arange(3.0)
    t = _tables(x, y, np.array([0.0, 1.0]), np.array([0.0, 1.0]))
    v = np.float32(37.1)
    cube = np.full((1, 2, 2), v, np.float32)
    w = oracle.boundary_edges(t, [cube] * 3, 0.01)[0]
    single = float(v * np.float32(0.01))
    assert single != float(v) * 0.01                    # the case tells the two apart
    assert w[0, 0, 0] == single


def test_missing_values_interpolate_as_zero():
    x, y = np.arange(3.0), np.arange(3.0)
    t = _tables(x, y, np.array([0.5, 1.0]), np.array([0.5, 1.0]))
    field = np.ones((1, 3, 3), np.float32)
    field[0, 0, 0] = -1.0e20
    cube = _footprint(t, field)
    assert cube.shape == (1, 2, 2)
    w = oracle.boundary_edges(t, [cube] * 3)[0]
    assert w[0, 0, 0] == 0.5 * (0.5 * 0.0 + 0.5 * 1.0) + 0.5 * 1.0   # west node at y = 0.5
    assert w[0, 0, 1] == 1.0                                          # y = 1: the row above only
