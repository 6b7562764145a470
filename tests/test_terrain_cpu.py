"""CPU checks of the oracle's terrain grains (shaders/world/terrain.wgsl):
hand-derived known answers for the sandpile slide, the stray walk of a lone
grain and grain_fall (with the eviction of the monomers that no longer fit),
and the reference's own invariants (tests/conservation.rs:207-250: terrain
changes and painting neither create nor destroy monomers)."""
import numpy as np
import pytest

import ribo_world as rw
from test_oracle_cpu import pcg4d_numpy

S_RELAX, S_SAND = 16, 32
# terrain.wgsl:294-303: the stray-walk directions
WALK = [(1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (-1, 1), (1, -1), (-1, -1)]


def u2f(u: int) -> float:
    return float(np.float32(u >> 8) * np.float32(1.0 / 16777216.0))


def _world(ro, n=16, seed=5, **params):
    o = ro.OracleWorld(n, seed=seed)
    z = np.zeros((n, n), np.uint32)
    o.upload(rw.GAMMA, z)
    o.upload(rw.CHEM, np.zeros((n, n, 4), np.uint32))
    o.settings.terrain_mode = 1
    o.params.sediment_settle = 0.0
    o.params.sediment_compaction = 0.0
    o.params.rock_crumble = 0.0
    o.params.dt = 1.0
    for k, v in params.items():
        setattr(o.params, k, v)
    return o


def test_sandpile_slide_known_answer(ro):
    """A lone rock cell (6 grains) on empty ground: its lowest neighbour is the
    first strictly lower of (x-1, x+1, y-1, y+1), i.e. x-1; it slides one grain
    there when rng_f4(idx, epoch, S_SAND + phase).x < 0.12 * max(settle, crumble)."""
    n, x, y = 16, 8, 8
    o = _world(ro, n, rock_crumble=1.0)
    idx = y * n + x
    moved = 0
    for epoch in range(120):
        g = np.zeros((n, n), np.uint32)
        g[y, x] = 6
        o.upload(rw.GAMMA, g)
        o.params.epoch = epoch
        o.run_pass(o.params, 16)  # relax pass a
        got = o.read(rw.GAMMA)
        want = g.copy()
        p = np.float32(0.12) * np.float32(1.0)
        if u2f(pcg4d_numpy([idx, epoch, S_SAND, o.params.seed])[0]) < p:
            want[y, x] = 5
            want[y, x - 1] = 1
            moved += 1
        assert np.array_equal(got, want), epoch
    assert 3 <= moved <= 40


def test_stray_walk_known_answer(ro):
    """A lone loose grain with no fluid, no vent and nothing around it: no
    current (p_sed = 0), mobility 0.25^0 = 1, no better nest (every score 0),
    so it walks in direction (rr.y >> 8) % 8 when (rr.z >> 8) / 2^24 < 0.05,
    rr = pcg4d(idx, epoch, S_RELAX + phase, seed)."""
    n, x, y = 16, 8, 8
    o = _world(ro, n, fluid_enabled=0)
    idx = y * n + x
    moved = 0
    for epoch in range(300):
        for phase in (0, 1):
            g = np.zeros((n, n), np.uint32)
            g[y, x] = 1
            o.upload(rw.GAMMA, g)
            o.params.epoch = epoch
            o.run_pass(o.params, 16 + phase)
            rr = pcg4d_numpy([idx, epoch, S_RELAX + phase, o.params.seed])
            want = g.copy()
            if u2f(rr[2]) < np.float32(0.05):
                dx, dy = WALK[(rr[1] >> 8) % 8]
                want[y, x] = 0
                want[y + dy, x + dx] = 1
                moved += 1
            assert np.array_equal(o.read(rw.GAMMA), want), (epoch, phase)
    assert 10 <= moved <= 60


def test_grain_fall_known_answer(ro):
    """grain_fall (terrain.wgsl:425-446): rock supports, a hole clears support,
    unsupported loose cells drop one row with all their grains, bottom-up; the
    fall clock ticks when floor(epoch * rf / 2^16) changes, rf = 0.5 * 2^16
    here (settle 1 -> 0.5 cells per step), i.e. on odd epochs.  A grain landing
    on a cell shrinks its capacity (48 -> 32 for one grain): the excess leaves,
    spent before activated, to the source cell, which now has room."""
    n, x = 16, 5
    o = _world(ro, n, sediment_settle=1.0)
    g = np.zeros((n, n), np.uint32)
    g[0, x], g[2, x], g[3, x], g[5, x] = 6, 1, 2, 1
    g[1, 9] = 2  # a supported-by-nothing cell in another column: y = 1 above a hole at y = 0
    chem = np.zeros((n, n, 4), np.uint32)
    chem[1, x, 0] = 30 | (10 << 16)  # 40 monomers where the first grain lands
    o.upload(rw.GAMMA, g)
    o.upload(rw.CHEM, chem)
    o.params.epoch = 0  # no tick
    o.run_pass(o.params, 18)
    assert np.array_equal(o.read(rw.GAMMA), g)
    o.params.epoch = 1
    o.run_pass(o.params, 18)
    want = g.copy()
    want[:6, x] = [6, 1, 2, 0, 1, 0]
    want[0, 9], want[1, 9] = 2, 0
    assert np.array_equal(o.read(rw.GAMMA), want)
    c = o.read(rw.CHEM)
    assert c[1, x, 0] == 30 | (2 << 16)  # 8 spent evicted: 32 = capacity with one grain
    assert c[2, x, 0] == 8 << 16          # to the source cell (then 2 grains: capacity 16 >= 8)
    assert int(c.sum()) == int(chem.sum())


def _channels(cells):
    led = rw.Ledger.from_cells(cells)
    return [led.channel(k) for k in range(4)]


def test_terrain_and_painting_conserve_matter(ro):
    """tests/conservation.rs:207-250 on the oracle: a rock block and a rubble
    band, a painted rock disc (its centre holds 6 grains), then 64 steps with
    the terrain block on: per-channel monomer totals never change, and the
    relax passes and grain_fall conserve the grains."""
    import synth

    n = 64
    o = ro.OracleWorld(n, seed=21)
    inp = synth.make_world_inputs(n, seed=21, rock_frac=0.0)
    gamma = np.zeros((n, n), np.uint32)
    gamma[n // 4:n // 2, n // 4:n // 2] = 6
    gamma[:n // 8, :] = np.where(gamma[:n // 8, :] == 0, 2, gamma[:n // 8, :])
    inp[rw.GAMMA] = gamma
    o.seed_inputs(inp)
    before = _channels(inp[rw.CHEM])
    o.encode_paint(n * 0.75, n * 0.75, 10.0, 6)
    g2 = o.read(rw.GAMMA)
    assert g2[n * 3 // 4, n * 3 // 4] == 6
    assert _channels(o.read_cells_blocking()) == before
    o.settings.terrain_mode = 1
    o.params.dt = 1.0
    o.params.sediment_settle = 0.6
    o.params.sediment_compaction = 0.3
    o.params.rock_crumble = 0.2
    o.params.sediment_threshold = 0.01
    grains = int(g2.sum())
    o.run(64)
    g3 = o.read(rw.GAMMA)
    assert int(g3.sum()) == grains
    assert (g3 != g2).sum() > 20, "the terrain did not move"
    assert _channels(o.read_cells_blocking()) == before


def test_relax_passes_conserve_with_vents_and_currents(ro):
    """Every branch of the loose-grain rule at once (compaction, shedding,
    currents, vent jets, the walk) over many relax passes: grains and
    monomers are conserved exactly and no count wraps."""
    import synth

    n = 48
    o = ro.OracleWorld(n, seed=9)
    inp = synth.make_world_inputs(n, seed=9, rock_frac=0.15, rubble_frac=0.35, max_disp=2.0)
    o.seed_inputs(inp)
    heat = np.zeros((n, n, 2), np.float32)
    heat[2:5, 20:26, 0] = 50.0
    o.upload(rw.HEAT, heat)
    o.settings.terrain_mode = 1
    for k, v in dict(dt=1.0, sediment_settle=0.8, sediment_compaction=0.5, rock_crumble=0.4,
                     sediment_threshold=0.001, sediment_transport=1.9).items():
        setattr(o.params, k, v)
    grains = int(inp[rw.GAMMA].sum())
    before = _channels(inp[rw.CHEM])
    for epoch in range(40):
        o.params.epoch = epoch
        for which in (16, 17, 18):
            o.run_pass(o.params, which)
    g = o.read(rw.GAMMA)
    assert int(g.sum()) == grains
    assert g.max() < 64
    assert (g != inp[rw.GAMMA]).sum() > 50
    assert _channels(o.read_cells_blocking()) == before
