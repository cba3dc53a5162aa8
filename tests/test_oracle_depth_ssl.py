"""The oracle's restatement of depth_ssl's setSSLim (depth_ssl/depth_ssl.f:
222-362) on hand-worked answers, and against a plain Python reading of the
same loops on random rough bathymetry.

The reference ships no data for this tool, so the known answers below are
worked by hand from the algorithm's statement.  They pin the two points a
restatement can get wrong:
- the scan along a line is in place: a node sees its left neighbour's new
  value;
- land (depth below depmin) blocks the open-water rule and drives the
  coastal rule, which needs land on exactly one side.
"""
import numpy as np
import pytest

import oracle


def test_spike_in_open_water():
    b, counts, st = oracle.depth_ssl(np.array([[100.0, 100.0, 1.0, 100.0, 100.0]]))
    assert np.array_equal(b, np.full((1, 5), 100.0))  # sqrt: 10 10 1 10 10 -> the mean 10
    assert counts[0] == 1 and counts[1] == 0 and st == 0


def test_spike_along_a_column():
    b, counts, st = oracle.depth_ssl(np.array([[100.0], [100.0], [1.0], [100.0], [100.0]]))
    assert np.array_equal(b, np.full((5, 1), 100.0))
    assert counts[0] == 1 and st == 0


def test_scan_is_in_place():
    # sqrt: 10 1 1 10.  Node 2: c2 = 10 > 2 -> (10 + 1) / 2 = 5.5.  Node 3 then
    # sees 5.5 on its left: c1 = 10 > 2 -> (5.5 + 10) / 2 = 7.75.  A
    # simultaneous update would give 5.5 twice.
    b, counts, st = oracle.depth_ssl(np.array([[100.0, 1.0, 1.0, 100.0]]))
    assert np.array_equal(b, np.array([[100.0, 30.25, 60.0625, 100.0]]))
    assert list(counts[:2]) == [2, 0] and st == 0


def test_coast_one_side_land():
    # node 2 is wet with land on its left only: at least 100 / alpha^2 = 25
    b, counts, st = oracle.depth_ssl(np.array([[0.05, 1.0, 100.0, 100.0]]))
    assert np.array_equal(b, np.array([[0.05, 25.0, 100.0, 100.0]]))
    assert counts[0] == 0 and counts[12] == 1 and counts[13] == 0 and st == 0


def test_coast_land_both_sides_and_depmin():
    # land on both sides: no coastal rule; 0.1 is not below depmin, so wet
    b, counts, _ = oracle.depth_ssl(np.array([[0.05, 1.0, 0.05, 0.1, 50.0]]))
    # node 4 (0.1) is wet with land on its left: at least 50 / 4 = 12.5
    assert np.array_equal(b, np.array([[0.05, 1.0, 0.05, 12.5, 50.0]]))
    assert counts[12] == 1


def test_alpha_changes_the_threshold():
    d = np.array([[100.0, 100.0, 9.0, 100.0, 100.0]])  # sqrt ratio 10/3 = 3.33
    b2, _, _ = oracle.depth_ssl(d, alpha=2.5)
    b3, _, _ = oracle.depth_ssl(d, alpha=3.5)
    assert b2[0, 2] == 100.0 and b3[0, 2] == 9.0


def _python_ssl(dep, alpha, depmin):
    """setSSLim read literally, in Python loops (small grids only)."""
    b = np.array(dep, dtype=np.float64)
    ny, nx = b.shape
    counts = []

    def lines():
        for i in range(nx):
            yield (slice(None), i)
        for j in range(ny):
            yield (j, slice(None))

    for _ in range(12):
        nodes = 0
        for sl in lines():
            q = list(b[sl])
            p = list(q)
            land = [v < depmin for v in q]
            q = [v if land[k] else np.sqrt(v) for k, v in enumerate(q)]
            for j in range(1, len(q) - 1):
                if not (land[j - 1] or land[j] or land[j + 1]):
                    if q[j + 1] / q[j] > alpha or q[j - 1] / q[j] > alpha:
                        q[j] = (q[j - 1] + q[j + 1]) / 2
                        p[j] = q[j] * q[j]
                        nodes += 1
            b[sl] = p
        counts.append(nodes)
        if nodes == 0:
            break
    a2 = alpha * alpha
    for _ in range(12):
        nodes = 0
        for sl in lines():
            q = list(b[sl])
            land = [v < depmin for v in q]
            for j in range(1, len(q) - 1):
                if not land[j] and (land[j + 1] != land[j - 1]):
                    dep = q[j - 1] if land[j + 1] else q[j + 1]
                    if dep / q[j] > a2:
                        q[j] = dep / a2
                        nodes += 1
            b[sl] = q
        counts.append(nodes)
        if nodes == 0:
            break
    return b


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_literal_reading(seed):
    rng = np.random.default_rng(seed)
    dep = np.exp(rng.uniform(-4.0, 8.0, (23, 31)))  # 0.02 m to 3000 m: land, coasts, rough water
    dep[rng.random(dep.shape) < 0.15] = -5.0
    got, counts, _ = oracle.depth_ssl(dep, 2.0, 0.1)
    ref = _python_ssl(dep, 2.0, 0.1)
    assert np.array_equal(got, ref)
    assert counts.sum() > 0
