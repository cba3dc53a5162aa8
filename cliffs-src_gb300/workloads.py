"""Seeded synthetic inputs with the shapes of the Cliffs benchmark workloads.

The reference ships no benchmark data (only two example archives), so these
generators stand in for its inputs.  Every case is a dict with the fields a
Cliffs run reads (cliffs_main.f, allabout.f):

  xcrd, ycrd   grid coordinates (m, or degrees when cartesian is False)
  cartesian    coordinate flag (allabout.f:23)
  dep          still-water depth (ny, nx) after bottom deformation, >0 water,
               rounded to float32 values so every arithmetic path starts from
               identical bathymetry
  H0           initial total water depth (ny, nx) before the celerity
               transform of cliffs_main.f:218-227 (cel = dep, plus the surface
               deformation, cliffs_main.f:193-212)
  u0, v0       initial velocities (ny, nx)
  ground, crough, dt, steps
  gauges       (I, J) 1-based node indices (allabout.f:83-89)
  gout, seaout output intervals in steps

Sizes, depths and sources follow the benchmark configurations: a 1-D channel
with a solitary wave running up a 1:20 beach, a 2-D shelf/slope basin with an
elliptical Gaussian uplift, and the same basin on a spherical grid.
"""
import numpy as np

GRAV = 9.800000190734863


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def channel_1d(seed=0, n=2000, dx=0.05, steps=5000):
    """1-D Cartesian channel: flat 1 m depth over the offshore 60 %, then a
    1:20 slope rising to +0.5 m of dry land (reached at x = 90 m), flat land
    to the end.  A sech^2 hump of amplitude A ~ U[0.02, 0.05] m (seeded),
    k = sqrt(3A/(4h^3)), centred 10 m offshore of the slope toe, u = 0.
    CFL 0.8 on the 1 m depth.  The coast is on the high-x side."""
    rng = np.random.default_rng(seed)
    x = np.arange(n, dtype=np.float64) * dx
    h = 1.0
    toe = 0.6 * n * dx
    dep = np.where(x < toe, h, h - (x - toe) / 20.0)
    dep = np.maximum(dep, -0.5)
    dep = _f32(dep).reshape(1, n)
    A = rng.uniform(0.02, 0.05)
    k = np.sqrt(3 * A / (4 * h ** 3))
    x0 = toe - 10.0
    eta0 = A / np.cosh(k * (x - x0)) ** 2
    H0 = dep + eta0.reshape(1, n)
    dt = 0.8 * dx / np.sqrt(GRAV * h)
    return dict(name="channel_1d", xcrd=x, ycrd=np.zeros(1), cartesian=True,
                dep=dep, H0=H0, u0=np.zeros((1, n)), v0=np.zeros((1, n)),
                ground=0.003, crough=0.0, dt=float(dt), steps=steps,
                gauges=(np.array([], np.int32), np.array([], np.int32)),
                gout=100, seaout=100, amplitude=float(A))


def _powerlaw_field(rng, ny, nx):
    """Random field with a k^-2 power spectrum, unit RMS."""
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    kk = np.sqrt(kx * kx + ky * ky)
    kk[0, 0] = 1.0
    amp = 1.0 / kk  # power ~ k^-2
    amp[0, 0] = 0.0
    ph = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    f = np.fft.irfft2(amp * ph, s=(ny, nx))
    return f / (f.std() + 1e-30)


def shelf_profile(xkm, length_km):
    """Cross-shore depth profile (m, >0 water) over a basin of the given
    length: 4000 m abyss, tanh shelf break to 200 m, 200 m shelf, then a
    linear slope reaching +50 m of land at the last column."""
    L = length_km
    brk = L - 26.8     # shelf-break centre
    s0 = L - 8.8       # start of the linear slope
    d = 200.0 + 1900.0 * (1.0 - np.tanh((xkm - brk) / 2.0))
    slope = 200.0 - 250.0 * (xkm - s0) / (L - s0)
    return np.where(xkm < s0, d, slope)


def shelf_2d(seed=0, nx=2048, ny=2048, dx=100.0, steps=3000, amp=2.0,
             axes_km=(100.0, 50.0), ngauges=64, perturb=0.05, centre_km=None):
    """2-D Cartesian basin, x cross-shore: 4000 m abyss, tanh shelf break to
    200 m, linear slope to +50 m land at the last columns, plus a k^-2 random
    perturbation of `perturb` x local |depth| (which also roughens the land).
    Source: elliptical Gaussian bottom uplift (full axes axes_km, amplitude
    amp, seeded orientation) applied instantaneously as in quake=1.
    Gauges at seeded wet nodes; dt from CFL 0.8 on the maximum depth."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx, dtype=np.float64) * dx
    y = np.arange(ny, dtype=np.float64) * dx
    Lkm = nx * dx / 1000.0
    d0 = shelf_profile(x / 1000.0, Lkm)[None, :].repeat(ny, 0)
    if perturb:
        d0 = d0 + perturb * np.abs(d0) * _powerlaw_field(rng, ny, nx)
    d0 = _f32(d0)
    theta = rng.uniform(0, np.pi)
    if centre_km is None:
        cx, cy = 0.45 * nx * dx, 0.5 * ny * dx
    else:
        cx, cy = centre_km[0] * 1000.0, centre_km[1] * 1000.0
    a, b = axes_km[0] * 500.0, axes_km[1] * 500.0  # half-axes in m
    X, Y = np.meshgrid(x - cx, y - cy)
    xr = X * np.cos(theta) + Y * np.sin(theta)
    yr = -X * np.sin(theta) + Y * np.cos(theta)
    uplift = amp * np.exp(-(xr / a) ** 2 - (yr / b) ** 2)
    # quake=1 (cliffs_main.f:193-207): cel = dep first, then dep -= uplift
    H0 = d0.copy()
    dep = _f32(d0 - uplift)
    hmax = float(np.max(d0))
    dt = 0.8 * dx / np.sqrt(GRAV * hmax)
    wet = np.argwhere(d0 > 10.0)
    pick = wet[rng.choice(len(wet), ngauges, replace=False)] if ngauges else np.zeros((0, 2), int)
    J = (pick[:, 0] + 1).astype(np.int32)
    I = (pick[:, 1] + 1).astype(np.int32)
    return dict(name=f"shelf_2d_{nx}x{ny}", xcrd=x, ycrd=y, cartesian=True,
                dep=dep, H0=H0, u0=np.zeros((ny, nx)), v0=np.zeros((ny, nx)),
                ground=0.01, crough=0.0, dt=float(dt), steps=steps,
                gauges=(I, J), gout=10, seaout=steps + 1, amplitude=float(amp),
                theta=float(theta))


EARTHR = 6371009.0  # earth radius of MasterGrid.f's metric


def sphere_2d(seed=3, nx=4320, ny=2160, lat=(-80.0, 80.0), dlon=1.0 / 12.0, steps=3000, ngauges=64,
              axes_nodes=(60, 30)):
    """shelf_2d laid out in node units (1 km per node) and placed on a
    spherical grid: longitudes 0, dlon, ... (nx nodes), latitudes evenly from
    lat[0] to lat[1] (ny nodes), cartesian False.  The source's full axes
    span axes_nodes nodes.  dt from CFL 0.8 on the smallest cell (the x
    spacing at the highest |latitude|) and the maximum depth."""
    case = shelf_2d(seed=seed, nx=nx, ny=ny, dx=1000.0, steps=steps, ngauges=ngauges,
                    axes_km=tuple(float(a) for a in axes_nodes))
    lon = np.arange(nx, dtype=np.float64) * dlon
    lats = np.linspace(lat[0], lat[1], ny)
    beta = np.pi * EARTHR / 180.0
    coslat = np.cos(np.radians(np.max(np.abs(lats))))
    dmin = min(beta * dlon * coslat, beta * (lats[1] - lats[0]))
    case.update(name=f"sphere_2d_{nx}x{ny}", xcrd=lon, ycrd=lats, cartesian=False,
                dt=float(0.8 * dmin / np.sqrt(GRAV * float(np.max(case["H0"])))))
    return case


def coast_profile(nx, land=16, slope=20, shelf=40):
    """Depth (m, > 0 water) across the columns of a basin whose coast runs
    along the east edge: `land` columns of land rising to +50 m at the edge, a
    slope of `slope` columns from the coast to 200 m, a shelf of `shelf`
    columns, then a tanh break (3 columns wide) to the 4000 m abyss (the
    shape of shelf_profile, in node units)."""
    s = (nx - 1 - land) - np.arange(nx, dtype=np.float64)  # columns seaward of the coast
    d = np.where(s < 0, 50.0 * s / land, 200.0 * np.minimum(s, slope) / slope)
    brk = slope + shelf
    return np.where(s > brk, 200.0 + 1900.0 * (1.0 + np.tanh((s - brk - 3.0) / 1.5)), d)


def _bilinear(x, y, f, xq, yq):
    """f (len(y), len(x)) at the points xq (m) x yq (n) of a lattice inside it."""
    i = np.clip(np.searchsorted(x, xq) - 1, 0, len(x) - 2)
    j = np.clip(np.searchsorted(y, yq) - 1, 0, len(y) - 2)
    tx = ((xq - x[i]) / (x[i + 1] - x[i]))[None, :]
    ty = ((yq - y[j]) / (y[j + 1] - y[j]))[:, None]
    f00, f10 = f[np.ix_(j, i)], f[np.ix_(j, i + 1)]
    f01, f11 = f[np.ix_(j + 1, i)], f[np.ix_(j + 1, i + 1)]
    return (1 - ty) * ((1 - tx) * f00 + tx * f10) + ty * ((1 - tx) * f01 + tx * f11)


def _wet_gauges(rng, dep, n, cols=None):
    """n seeded wet nodes (depth > 10 m), optionally within a column range."""
    mask = dep > 10.0
    if cols is not None:
        keep = np.zeros_like(mask)
        keep[:, cols[0]:cols[1]] = True
        mask &= keep
    wet = np.argwhere(mask)
    pick = wet[rng.choice(len(wet), min(n, len(wet)), replace=False)]
    return (pick[:, 1] + 1).astype(np.int32), (pick[:, 0] + 1).astype(np.int32)


def nested_sphere(seed=3, nx=4320, ny=2160, lat=(-80.0, 80.0), dlon=1.0 / 12.0, sizes=(600, 900), ratio=3,
                  land=16, slope=5, shelf=12, ngauges=64, source_km=2000.0, half_km=(75.0, 30.0), amp=3.0,
                  perturb=0.05, dwall=5.0, ground=0.1):
    """A spherical master grid with a chain of one-way nested children, each
    at refinement `ratio` inside the previous one (NestedGrid.f), shaped like
    the 1/12 degree, 4320 x 2160 benchmark configuration.

    The master has the coast along its east edge (coast_profile with land,
    slope and shelf in master columns, plus a k^-2 perturbation of `perturb`
    x |depth|).  Each child is a square of
    sizes[k] nodes at 1/ratio of its parent's spacing.  Its east edge lies on
    land, `land` // 2 master columns (less at deeper levels) inside the master's
    edge, so every child holds a stretch of coast.  Rows are centred at 65 %
    of the master's latitude range.  A child's depth is its parent's,
    interpolated bilinearly.  Every grid starts at rest; the source is a
    dipole (amp = +3 m uplift, a -1 m trough two half-widths away, e-folding
    half-widths half_km = 75 km x 30 km, i.e. 150 km x 60 km) centred
    `source_km` west of
    the coast at the children's latitude, to be applied to every level by
    cliffs_gpu_add_source as a bottom deformation.

    ground (the minimal flow depth) is 0.1 m: the explicit friction term
    g n^2 u |u| / H^1.5 (cliffs.f:204) is stable for dt g n^2 |u| / H^1.5 < 2,
    which at the innermost grid's dt of ~3 s and ground = 0.01 m fails for
    |u| above 0.1 m/s in a newly flooded cell.

    Land inundation (runup) is on in the innermost grid only.  The outer
    grids have a vertical wall instead, as cliffs_main.f:131-137 makes it for
    itopo = 0: every cell shallower than dwall is set to -999 m, land that
    never floods.  Children are interpolated from their parent's depth before
    the wall.

    Returns (levels, source).  levels[k] is a case dict (xcrd, ycrd in degrees,
    cartesian False, dep, H0 = dep, u0, v0, ground, crough, dt, gauges, runup);
    the children's dt is the parent's divided by ratio.  source holds the keyword
    arguments of GpuGrid.add_source except the coordinates."""
    rng = np.random.default_rng(seed)
    lon = np.arange(nx, dtype=np.float64) * dlon
    lats = np.linspace(lat[0], lat[1], ny)
    d0 = coast_profile(nx, land, slope, shelf)[None, :].repeat(ny, 0)
    if perturb:
        d0 = d0 + perturb * np.abs(d0) * _powerlaw_field(rng, ny, nx)
    dep = _f32(d0)
    beta = np.pi * EARTHR / 180.0
    coslat = np.cos(np.radians(np.max(np.abs(lats))))
    dmin = min(beta * dlon * coslat, beta * (lats[1] - lats[0]))
    dt = float(0.8 * dmin / np.sqrt(GRAV * float(np.max(dep))))
    levels = [dict(name=f"master_{nx}x{ny}", xcrd=lon, ycrd=lats, cartesian=False, dep=dep, H0=dep.copy(),
                   u0=np.zeros_like(dep), v0=np.zeros_like(dep), ground=ground, crough=0.000625, dt=dt,
                   gauges=_wet_gauges(rng, dep, ngauges))]
    lat_c = lats[0] + 0.65 * (lats[-1] - lats[0])
    east = lon[nx - 1 - land // 2]  # every child's east edge: on the master's land
    for k, n in enumerate(sizes):
        p = levels[-1]
        sx = (p["xcrd"][1] - p["xcrd"][0]) / ratio
        sy = (p["ycrd"][1] - p["ycrd"][0]) / ratio
        e = east - (k * max(land // 4, 1)) * dlon  # deeper levels stop a little further west
        x = e - sx * np.arange(n - 1, -1, -1, dtype=np.float64)
        y = lat_c + sy * (np.arange(n, dtype=np.float64) - (n - 1) / 2.0)
        dk = _f32(_bilinear(p["xcrd"], p["ycrd"], p["dep"], x, y))
        coast = int(np.argmax(dk[n // 2] < 0.0)) if (dk[n // 2] < 0.0).any() else n
        levels.append(dict(name=f"child{k + 1}_{n}x{n}", xcrd=x, ycrd=y, cartesian=False, dep=dk,
                           H0=dk.copy(), u0=np.zeros_like(dk), v0=np.zeros_like(dk), ground=ground,
                           crough=0.000625, dt=p["dt"] / ratio,
                           gauges=_wet_gauges(rng, dk, ngauges, cols=(max(coast - 60, 0), coast))))
    for c in levels[:-1]:  # walls on every grid but the innermost
        c["dep"] = np.where(c["dep"] <= dwall, -999.0, c["dep"])
        c["H0"] = c["dep"].copy()
        c["runup"] = False
    levels[-1]["runup"] = True
    x0 = east - land * dlon - source_km / (beta / 1000.0 * np.cos(np.radians(lat_c)))
    source = dict(x0=float(x0), y0=float(lat_c),
                  ax=float(half_km[0] / (beta / 1000.0 * np.cos(np.radians(lat_c)))),
                  ay=float(half_km[1] / (beta / 1000.0)), angle=float(rng.uniform(-0.5, 0.5) + np.pi / 2),
                  amp=float(amp), dipole=1.0 / 3.0, bottom=1)
    return levels, source
