"""Seeded synthetic world inputs (stand-ins for the reference's seeded worlds).

Generates the state the world step starts from, with the shapes and value
distributions of the benchmark configurations:
  * velocity (u, v) f32 at fluid resolution: 4-octave value noise
    (persistence 0.5, smoothstep interpolation, lattice values from a
    SplitMix64 hash of the seed), scaled so that the largest speed moves
    `max_disp` environment cells per step at the given dt; zero in walls;
  * obstacles: gamma = 6 (rock) where an independent value-noise field
    exceeds its (1 - rock_frac) quantile, else 0;
  * monomers: 8 counts per cell ~ Poisson(monomer_mean) (A U G C x
    activated / spent), packed as act | spent << 16 into 4 u32, 0 in rock;
  * UV light (two bands at half resolution): exponential depth profile;
  * temperature, redox, vent heat: zero.
"""
from __future__ import annotations

import numpy as np

try:  # package-relative when imported as part of the package
    from . import ribo_world as rw
except ImportError:  # flat import from the package directory
    import ribo_world as rw

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea & Flood 2014) applied elementwise."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def _lattice(seed: int, octave: int, ix: np.ndarray, iy: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        k = (np.uint64(seed) * np.uint64(0x632BE59BD9B4E019)) ^ (np.uint64(octave + 1) * np.uint64(0x9E3779B97F4A7C15))
        h = _splitmix(k ^ (ix.astype(np.uint64) * np.uint64(0xD6E8FEB86659FD93)) ^ (iy.astype(np.uint64) * np.uint64(0xCA5A826395121157)))
    return (h >> np.uint64(40)).astype(np.float64) / float(1 << 24)


def value_noise(w: int, h: int, seed: int, octaves: int = 4, base_period: float = 64.0, persistence: float = 0.5) -> np.ndarray:
    """Fractal value noise in [0, 1], shape (h, w), float32.

    The lattice values are hashed once per lattice point and gathered per
    cell (the same values as hashing per cell)."""
    xs = np.arange(w, dtype=np.float64)[None, :]
    ys = np.arange(h, dtype=np.float64)[:, None]
    out = np.zeros((h, w))
    amp, norm, period = 1.0, 0.0, base_period
    for o in range(octaves):
        px, py = xs / period, ys / period
        ix, iy = np.floor(px), np.floor(py)
        tx, ty = px - ix, py - iy
        sx, sy = tx * tx * (3 - 2 * tx), ty * ty * (3 - 2 * ty)
        ix, iy = ix.astype(np.int64), iy.astype(np.int64)
        lx = np.arange(int(ix.max()) + 2, dtype=np.int64)[None, :]
        ly = np.arange(int(iy.max()) + 2, dtype=np.int64)[:, None]
        lat = _lattice(seed, o, lx, ly)  # lat[j, i] = lattice value at (i, j)
        a = lat[iy, ix]
        b = lat[iy, ix + 1]
        c = lat[iy + 1, ix]
        d = lat[iy + 1, ix + 1]
        v = (a + (b - a) * sx) * (1 - sy) + (c + (d - c) * sx) * sy
        out += amp * v
        norm += amp
        amp *= persistence
        period /= 2.0
    return (out / norm).astype(np.float32)


def make_world_inputs(grid, fluid=None, seed: int = 1000, rock_frac: float = 0.10, monomer_mean: float = 4.0,
                      max_disp: float = 0.5, dt: float = 1.0, uv_depth: float = 2.0, rubble_frac: float = 0.0) -> dict:
    """Returns {ribo_world field id: numpy array} for a world of the given size.
    rubble_frac > 0 turns that fraction of the non-rock cells into rubble (1 or 2 grains)."""
    gw, gh = (grid, grid) if isinstance(grid, int) else grid
    fw, fh = (gw, gh) if fluid is None else ((fluid, fluid) if isinstance(fluid, int) else fluid)
    r = gw // fw
    rng = np.random.Generator(np.random.PCG64(seed))
    # obstacles
    rn = value_noise(gw, gh, seed * 7 + 1, octaves=4, base_period=max(8.0, min(gw, gh) / 8.0))
    thr = np.quantile(rn, 1.0 - rock_frac) if rock_frac > 0 else np.inf
    gamma = np.where(rn > thr, 6, 0).astype(np.uint32)
    if rubble_frac > 0:
        rr = rng.random((gh, gw))
        rub = (rr < rubble_frac) & (gamma == 0)
        gamma[rub] = np.where(rr[rub] < rubble_frac / 2, 1, 2).astype(np.uint32)
    # monomers: 8 Poisson counts per cell
    counts = rng.poisson(monomer_mean, size=(gh, gw, 4, 2)).astype(np.uint32)
    counts = np.minimum(counts, 0xFFFF)
    counts[gamma >= 3] = 0
    chem = (counts[..., 0] | (counts[..., 1] << 16)).astype(np.uint32)
    # velocity at fluid resolution, zero where the fluid cell is mostly rock
    u = value_noise(fw, fh, seed * 7 + 2) * 2 - 1
    v = value_noise(fw, fh, seed * 7 + 3) * 2 - 1
    vel = np.stack([u, v], axis=-1).astype(np.float64)
    speed = np.sqrt((vel ** 2).sum(-1)).max()
    vmax = max_disp / (max(dt, 1e-6) * r)
    vel *= vmax / max(speed, 1e-12)
    rock_f = gamma.reshape(fh, r, fw, r).max(axis=(1, 3)) >= 3
    vel[rock_f] = 0
    # UV light: exponential fall-off with depth, two bands
    lw, lh = gw // 2, gh // 2
    depth = (lh - 1 - np.arange(lh)) / lh
    band0 = np.exp(-uv_depth * depth)[:, None] * np.ones((1, lw))
    band1 = np.exp(-uv_depth * 0.03 * depth)[:, None] * np.ones((1, lw))
    light = np.stack([band0, band1]).astype(np.float32)
    zf = np.zeros((fh, fw), np.float32)
    return {
        rw.GAMMA: gamma,
        rw.CHEM: chem,
        rw.VELOCITY: vel.astype(np.float32),
        rw.LIGHT: light,
        rw.PRESSURE: zf,
        rw.TEMP: zf,
        rw.REDOX: zf,
    }


def bench_params(seed: int = 1000, defaults=None) -> "rw.SimParams":
    """SimParams of the benchmark workload: reference defaults, dt = 1,
    sun heating off, every step a full fluid + transport step.

    `defaults(seed)` supplies the reference defaults; the library's own
    table by default.  A caller that must not load the CUDA library (a
    CPU-only measurement) passes a table of its own."""
    p = (defaults or rw.default_params)(seed)
    p.dt = 1.0
    p.sun_heat = 0.0
    p.transport_every = 1
    p.day_period = 0.0
    return p


# The batched workload: worlds of uneven sizes drawn by seed from these
# grids (square sides, then two rectangles), each with its own noise seed,
# obstacle fraction U(0.05, 0.25) and monomer mean U(1, 8).
BATCH_GRIDS = [(s, s) for s in (128, 192, 256, 384, 512, 768, 1024)] + [(512, 2048), (2048, 256)]


def batch_specs(n: int = 64, seed: int = 7):
    """[(grid (w, h), noise seed, rock_frac, monomer_mean)] of the batched workload."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        g = BATCH_GRIDS[int(rng.integers(len(BATCH_GRIDS)))]
        out.append((g, 1000 + i, float(rng.uniform(0.05, 0.25)), float(rng.uniform(1.0, 8.0))))
    return out
