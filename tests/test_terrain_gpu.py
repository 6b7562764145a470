"""Parity of the terrain grains (terrain_mode 1: relax passes, grain_fall, the
slope, the wall mask rebuilt every fluid step) and of the terrain brush with
the CPU oracle, bit for bit, through the C ABI."""
import numpy as np
import pytest

from helpers import STATE_FIELDS, assert_same, compare_worlds, setup_pair

pytestmark = pytest.mark.gpu

BASE = dict(dt=1.0, transport_every=1, sun_heat=0.0, day_period=0.0)
ACTIVE = dict(BASE, sediment_settle=0.6, sediment_compaction=0.3, rock_crumble=0.3, sediment_threshold=0.01)

CASES = [
    # id, grid, fluid, params, settings, steps, synth
    ("reference-defaults-rubble", 96, None, BASE, dict(fluid_substep=1, terrain_mode=1), 8,
     dict(rubble_frac=0.3)),
    ("active-grains-vents", 128, None, ACTIVE, dict(fluid_substep=1, terrain_mode=1), 10,
     dict(rubble_frac=0.3, rock_frac=0.15, max_disp=2.0)),
    ("substep-2-half-fluid", 128, 64, ACTIVE, dict(fluid_substep=2, terrain_mode=1), 9,
     dict(rubble_frac=0.25)),
    ("rect-160x96-crowded", (160, 96), None, dict(ACTIVE, settle=2.0), dict(fluid_substep=1, terrain_mode=1), 8,
     dict(rubble_frac=0.4, monomer_mean=12.0)),
    ("jacobi-fall-every-step", 64, None, dict(ACTIVE, sediment_settle=1.0, dt=2.0),
     dict(fluid_substep=1, terrain_mode=1, multigrid=0, jacobi_iters=8), 8, dict(rubble_frac=0.5, dt=2.0)),
    # sides that are not multiples of the 32-cell warp rows or of the 3 x 3 classes
    ("ragged-100x74-half-fluid", (100, 74), (50, 37), dict(ACTIVE, sediment_settle=1.0), dict(fluid_substep=1, terrain_mode=1),
     8, dict(rubble_frac=0.35)),
]

FIELDS = STATE_FIELDS


def _vents(rw, g, o):
    heat = np.zeros(g.field_shape(rw.HEAT)[0], np.float32)
    fh, fw = heat.shape[:2]
    heat[2:5, fw // 3:fw // 3 + 6, 0] = 30.0
    heat[2:5, fw // 3:fw // 3 + 6, 1] = 5.0
    g.upload(rw.HEAT, heat)
    o.upload(rw.HEAT, heat)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_terrain_steps_bit_exact(rw, ro, case):
    _, grid, fluid, params, settings, steps, syn = case
    g, o, inputs = setup_pair(rw, ro, grid, fluid, params=params, settings=settings, **syn)
    _vents(rw, g, o)
    done = 0
    for batch in (1, 2, steps - 3):
        g.encode_steps(batch)
        o.encode_steps(batch)
        done += batch
        compare_worlds(g, o, f"{case[0]} after {done} steps", FIELDS)
    gam = g.read(rw.GAMMA)
    assert int(gam.sum()) == int(inputs[rw.GAMMA].sum()), "grains are conserved"
    if params is not BASE:
        assert (gam != inputs[rw.GAMMA]).sum() > 0, "the terrain moved"
    assert g.ledger_blocking() == o.ledger_blocking()


def test_paint_then_terrain_steps(rw, ro):
    """The brush (World::encode_paint) on a frozen terrain and then with the
    terrain block on: gamma, the evicted monomers, the slope and the mask
    match the oracle; per-channel totals are unchanged
    (tests/conservation.rs:240-249)."""
    g, o, inputs = setup_pair(rw, ro, 96, params=ACTIVE, settings=dict(fluid_substep=1), rubble_frac=0.2,
                              monomer_mean=8.0)
    before = rw.Ledger.from_cells(inputs[rw.CHEM])
    for w in (g, o):
        w.encode_paint(72.0, 72.0, 10.0, 6)
    compare_worlds(g, o, "after the brush", FIELDS)
    assert g.read(rw.GAMMA)[72, 72] == 6
    g.encode_steps(2)
    o.encode_steps(2)
    compare_worlds(g, o, "frozen terrain after the brush", FIELDS)
    for w in (g, o):
        w.settings.terrain_mode = 1
        w.encode_paint(20.5, 30.0, 6.5, 2)
        w.encode_paint(0.0, 95.0, 5.0, 4)  # a disc cut by the world's corner
    g.encode_steps(4)
    o.encode_steps(4)
    compare_worlds(g, o, "terrain steps after the brush", FIELDS)
    after = g.ledger_blocking()
    assert [after.channel(k) for k in range(4)] == [before.channel(k) for k in range(4)]


def test_terrain_graph_replay(rw, ro):
    """Step sequences with the terrain block replay from CUDA graphs (the
    grain_fall launches are part of the key): 6 calls of 4 steps (the key
    alternates with the parameter slot: calls 2 and 3 are captured, 4 and 5
    replayed) equal the oracle."""
    g, o, _ = setup_pair(rw, ro, 96, params=ACTIVE, settings=dict(fluid_substep=1, terrain_mode=1), rubble_frac=0.3)
    for k in range(6):
        g.encode_steps(4)
        o.encode_steps(4)
        compare_worlds(g, o, f"call {k}", FIELDS)


def test_terrain_rejected_where_it_cannot_run(rw):
    """Batches and the mixed-precision solver take a frozen terrain."""
    import synth

    w = rw.World(128, seed=3, mg_min_size=16, precision_mode=1)  # RIBO_PRECISION_MIXED
    w.seed_inputs(synth.make_world_inputs(128, seed=3))
    w.settings.terrain_mode = 1
    with pytest.raises(rw.RiboError, match="frozen terrain"):
        w.encode_steps(1)
    a = rw.World(64, seed=3)
    a.seed_inputs(synth.make_world_inputs(64, seed=3))
    a.settings.terrain_mode = 1
    b = rw.Batch()
    b.add(a)
    a._sync_settings()
    with pytest.raises(rw.RiboError, match="terrain_mode 0"):
        b.encode_steps(1)
