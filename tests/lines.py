"""Seeded generators of adversarial grid lines for the line-solver tests.

Values are drawn from small sets that straddle every decision of the
reference's wet/dry logic (cliffs.f:56-122, 264-329): land vs water around
celmin, both flooding criteria, transcritical flow for the sonic branch,
land/water edges, and fully dry lines.  Depths are float32-exact so the FP32
GPU path and the FP64 oracle start from identical bathymetry.
"""
import numpy as np

GRAV = 9.800000190734863


def random_grid(rng, nlines, n, ground=0.01, exact_thresholds=True, dry_frac=0.1):
    """Return (dep, cel, u, v) of shape (nlines + 2, n) for an x-sweep test.

    Rows 0 and nlines+1 are the untouched border rows of a 2-D grid.
    exact_thresholds puts celerities exactly on celmin (useful for the FP64
    equivalence tests, avoided for FP32-vs-FP64 comparisons).
    """
    celmin = np.sqrt(GRAV * ground)
    ny = nlines + 2
    d_set = np.array([-0.5, -0.05, 0.005, 0.02, 0.3, 1.0, 2.0, 5.0], np.float32)
    dep = d_set[rng.integers(0, len(d_set), (ny, n))].astype(np.float64)
    dep += rng.uniform(-0.004, 0.004, (ny, n)).astype(np.float32)
    dep = dep.astype(np.float32).astype(np.float64)
    if exact_thresholds:
        h_set = np.array([0.0, 0.5 * celmin, celmin, 1.01 * celmin, 0.5, 1.0, 3.0, 4.4])
    else:
        h_set = np.array([0.0, 0.5 * celmin, 0.97 * celmin, 1.05 * celmin, 0.5, 1.0, 3.0, 4.4])
    cel = h_set[rng.integers(0, len(h_set), (ny, n))]
    wet = cel > celmin
    # a wet cell is usually consistent with its depth: H near dep
    Hc = np.maximum(dep, 0) + rng.uniform(-0.02, 0.3, (ny, n))
    smooth = wet & (rng.random((ny, n)) < 0.5) & (Hc > ground * 1.5)
    cel = np.where(smooth, np.sqrt(GRAV * np.maximum(Hc, 0)), cel)
    u_set = np.array([-3.0, -0.5, -0.0, 0.0, 0.5, 3.0])
    u = u_set[rng.integers(0, len(u_set), (ny, n))] * rng.uniform(0.5, 1.5, (ny, n))
    v = rng.choice([-1.0, 0.0, 1.0], (ny, n)) * rng.uniform(0.5, 1.5, (ny, n))
    dry_rows = rng.random(ny) < dry_frac
    cel[dry_rows] = np.where(rng.random((dry_rows.sum(), n)) < 0.5, 0.0, 0.5 * celmin)
    return dep, cel, u, v


def random_spacing(rng, n, lo=0.5, hi=2.0):
    return rng.uniform(lo, hi, n - 1)
