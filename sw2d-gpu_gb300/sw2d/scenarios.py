"""Seeded synthetic scenarios with the shapes, sizes and value distributions of
the benchmark configurations (no dataset is shipped with the reference for
them, so they are generated here; every generator takes a seed).

All rasters are float64, row-major, north row first; x grows with the column,
y with the row (southwards).
"""
from __future__ import annotations

import numpy as np

MANNING_CLASSES = (0.03, 0.05, 0.08, 0.12)


def dam_break_channel(rows=256, cols=512, dx=1.0, h_up=10.0, x_gate=256.0):
    """1D-in-2D dam break on a flat frictionless channel: z = 0, depth h_up
    for x < x_gate and dry downstream, reflective walls."""
    z = np.zeros((rows, cols))
    x = (np.arange(cols) + 0.5) * dx
    h = np.where(x < x_gate, h_up, 0.0)[None, :].repeat(rows, axis=0)
    return {"z": z, "h0": h, "n": None, "dx": dx, "manning": 0.0}


def _value_noise(rng, rows, cols, octaves=6, persistence=0.5, base=4):
    """Fractal value noise in [-1, 1] (sum of bilinearly interpolated random
    lattices, frequency doubling per octave)."""
    out = np.zeros((rows, cols))
    amp, total = 1.0, 0.0
    yi = np.linspace(0.0, 1.0, rows)
    xi = np.linspace(0.0, 1.0, cols)
    for o in range(octaves):
        f = base * (2 ** o)
        lat = rng.uniform(-1.0, 1.0, size=(f + 1, f + 1))
        gy, gx = yi * f, xi * f
        iy = np.minimum(gy.astype(np.int64), f - 1)
        ix = np.minimum(gx.astype(np.int64), f - 1)
        wy = (gy - iy)[:, None]
        wx = (gx - ix)[None, :]
        a = lat[iy][:, ix]
        b = lat[iy][:, ix + 1]
        c = lat[iy + 1][:, ix]
        d = lat[iy + 1][:, ix + 1]
        out += amp * ((a * (1 - wx) + b * wx) * (1 - wy) + (c * (1 - wx) + d * wx) * wy)
        total += amp
        amp *= persistence
    return out / total


def _carve_channel(z, width=3, depth=1.0, drop=1e-3):
    """Carves a channel `width` cells wide along the steepest southward D8
    descent from the north-edge midpoint to the south edge, lowered by
    `depth` and made monotone (non-increasing) downstream."""
    rows, cols = z.shape
    j = cols // 2
    path = []
    for i in range(rows):
        path.append((i, j))
        if i + 1 < rows:
            cand = [(z[i + 1, jj], jj) for jj in (j - 1, j, j + 1) if 1 <= jj < cols - 1]
            j = min(cand)[1]
    level = None
    half = width // 2
    for (i, j) in path:
        lo = max(0, j - half)
        hi = min(cols, j + half + 1)
        v = z[i, lo:hi].min() - depth
        if level is not None and v > level - drop:
            v = level - drop
        z[i, lo:hi] = v
        level = v
    return z


def _voronoi_classes(rng, rows, cols, n_sites=256, classes=MANNING_CLASSES):
    sites = np.column_stack([rng.uniform(0, rows, n_sites), rng.uniform(0, cols, n_sites)])
    cls = rng.integers(0, len(classes), size=n_sites)
    vals = np.asarray(classes)[cls]
    try:
        from scipy.spatial import cKDTree
        ii, jj = np.mgrid[0:rows, 0:cols]
        pts = np.column_stack([ii.ravel() + 0.5, jj.ravel() + 0.5])
        _, idx = cKDTree(sites).query(pts)
        return vals[idx].reshape(rows, cols)
    except ImportError:  # numpy fallback, row by row
        out = np.empty((rows, cols))
        jc = np.arange(cols) + 0.5
        for i in range(rows):
            d = (sites[:, 0:1] - (i + 0.5)) ** 2 + (sites[:, 1:2] - jc[None, :]) ** 2
            out[i] = vals[np.argmin(d, axis=0)]
        return out


def catchment(n=2048, dx=5.0, seed=0, slope=0.01, amplitude=2.0, persistence=0.5, octaves=6,
              channel=True, manning="voronoi", manning_scale=1.0, cols=None):
    """Synthetic catchment: a plane tilted toward the south edge (slope), plus
    seeded fractal noise (octaves, amplitude, persistence), a 3-cell channel
    along the steepest southward descent, and Manning n from 4 land-use
    classes by seeded Voronoi patches (or a scalar when manning is a float).
    Starts dry."""
    rows = n
    cols = n if cols is None else cols
    rng = np.random.default_rng(np.random.PCG64(seed))
    i = np.arange(rows)[:, None]
    z = slope * dx * (rows - 1 - i) + np.zeros((1, cols))
    z = z + amplitude * _value_noise(rng, rows, cols, octaves=octaves, persistence=persistence)
    if channel:
        z = _carve_channel(z)
    if isinstance(manning, str):
        nm = _voronoi_classes(rng, rows, cols) * manning_scale
        scalar = 0.0
    else:
        nm = None
        scalar = float(manning) * manning_scale
    return {"z": z, "h0": np.zeros((rows, cols)), "n": nm, "dx": dx, "manning": scalar}


def triangular_hyetograph(peak_mm_h, duration_s):
    """Knots (mm/h) of a triangular hyetograph for RAIN_LINEAR: 0 at t=0,
    peak at duration/2, 0 at duration; knot spacing duration/2."""
    return np.array([0.0, float(peak_mm_h), 0.0]), duration_s / 2.0


class TerrainBank:
    """Scenario terrains cut from one seeded master catchment.

    Generating a fresh fractal DEM per scenario costs seconds at 1024^2; an
    ensemble or a request stream instead takes seeded random windows of one
    master catchment (same slope, noise statistics and Voronoi roughness
    classes), so each scenario still has its own terrain."""

    def __init__(self, size=2048, dx=5.0, seed=0):
        self.master = catchment(size, dx=dx, seed=seed)
        self.size, self.dx = size, dx

    def crop(self, side, rng, manning_scale=1.0):
        side = min(int(side), self.size)
        i0 = int(rng.integers(0, self.size - side + 1))
        j0 = int(rng.integers(0, self.size - side + 1))
        z = np.ascontiguousarray(self.master["z"][i0:i0 + side, j0:j0 + side])
        n = np.ascontiguousarray(self.master["n"][i0:i0 + side, j0:j0 + side]) * manning_scale
        return {"z": z, "h0": np.zeros((side, side)), "n": n, "dx": self.dx}


def ensemble(bank, count=256, sides=(128, 256, 512, 1024), seed=1, tail=1800.0):
    """The batched-ensemble configuration: sides uniform over `sides`, each
    scenario with a triangular hyetograph (peak U[20,120] mm/h, duration
    U[900,3600] s) and a Manning scaling U[0.8,1.2]; horizon = duration +
    `tail` seconds (the configuration does not give one)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        side = int(rng.choice(sides))
        peak = float(rng.uniform(20.0, 120.0))
        dur = float(rng.uniform(900.0, 3600.0))
        s = bank.crop(side, rng, manning_scale=float(rng.uniform(0.8, 1.2)))
        knots, kdt = triangular_hyetograph(peak, dur)
        s.update(rain=knots, rain_dt=kdt, t_end=dur + tail, side=side)
        out.append(s)
    return out


def request_stream(bank, rate, count, seed=2, side_min=64, side_max=2048, horizon=(600.0, 7200.0)):
    """The served-stream configuration: Poisson arrivals at `rate`/s, grid
    side log-uniform over [side_min, side_max] rounded to a multiple of 32,
    simulated horizon uniform over `horizon`, triangular rain as above."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    out = []
    for k in range(count):
        side = float(np.exp(rng.uniform(np.log(side_min), np.log(side_max))))
        side = int(max(32, min(side_max, 32 * round(side / 32))))
        h_end = float(rng.uniform(*horizon))
        peak = float(rng.uniform(20.0, 120.0))
        dur = float(rng.uniform(900.0, 3600.0))
        s = bank.crop(side, rng, manning_scale=float(rng.uniform(0.8, 1.2)))
        knots, kdt = triangular_hyetograph(peak, dur)
        s.update(rain=knots, rain_dt=kdt, t_end=h_end, side=side, arrival=float(t[k]))
        out.append(s)
    return out
