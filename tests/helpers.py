"""Shared helpers for the parity tests."""
import numpy as np

import ribo_world as rw

# Fields compared after a step: (field id, name).
STATE_FIELDS = [
    (rw.CHEM, "chem"), (rw.VELOCITY, "velocity"), (rw.PRESSURE, "pressure"), (rw.TEMP, "temperature"),
    (rw.REDOX, "redox"), (rw.DIVERGENCE, "divergence"), (rw.VEL_SMOOTH, "velocity_smooth"),
    (rw.NET_FLUX, "net_flux"), (rw.SOLID_MASK, "solid_mask"), (rw.SLOPE, "slope"),
    (rw.FORCE_VECTORS, "force_vectors"), (rw.REDOX_EATEN, "redox_eaten"), (rw.LIGHT, "light"),
    (rw.GAMMA, "gamma"),
]


def bits(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_same(a: np.ndarray, b: np.ndarray, what: str):
    """Bit-exact equality; on failure reports the first differing index."""
    ab, bb = bits(a).reshape(-1), bits(b).reshape(-1)
    if ab.shape != bb.shape:
        raise AssertionError(f"{what}: shapes {a.shape} vs {b.shape}")
    diff = np.nonzero(ab != bb)[0]
    if diff.size:
        i = diff[0]
        fa, fb = a.reshape(-1)[i], b.reshape(-1)[i]
        raise AssertionError(f"{what}: {diff.size} of {ab.size} words differ; first at {i}: {fa!r} vs {fb!r}")


def compare_worlds(gpu, orc, what: str, fields=STATE_FIELDS):
    for f, name in fields:
        assert_same(gpu.read(f), orc.read(f), f"{what}: {name}")


def setup_pair(rw_mod, ro_mod, grid, fluid=None, seed=1000, inputs=None, mg_min_size=8, mg_pre=2, mg_post=2,
               mg_coarse=30, params=None, settings=None, **synth_kw):
    import synth

    g = rw_mod.World(grid, fluid, seed=seed, mg_min_size=mg_min_size, mg_pre=mg_pre, mg_post=mg_post,
                     mg_coarse=mg_coarse)
    o = ro_mod.OracleWorld(grid, fluid, seed=seed, mg_min_size=mg_min_size, mg_pre=mg_pre, mg_post=mg_post,
                           mg_coarse=mg_coarse)
    if inputs is None:
        inputs = synth.make_world_inputs(grid, fluid, seed=seed, **synth_kw)
    g.seed_inputs(inputs)
    o.seed_inputs(inputs)
    for k, v in (params or {}).items():
        setattr(g.params, k, v)
        setattr(o.params, k, v)
    for k, v in (settings or {}).items():
        setattr(g.settings, k, v)
        setattr(o.settings, k, v)
    return g, o, inputs
