"""Parity of the CUDA world step with the CPU oracle (bit-exact), through the
C ABI.  Mirrors the reference's world tests (tests/conservation.rs) and adds
field-by-field comparisons after every batch of steps."""
import numpy as np
import pytest

from helpers import assert_same, compare_worlds, setup_pair

pytestmark = pytest.mark.gpu


BASE = dict(dt=1.0, transport_every=1, sun_heat=0.0, day_period=0.0)

CASES = [
    # id, grid, fluid, params, settings, steps, mg
    ("c0-256-mg5-2x3+3", 256, None, BASE, dict(fluid_substep=1, mg_cycles=2), 6, dict(mg_min_size=16, mg_pre=3, mg_post=3)),
    ("c0-256-unfused-dispatch", 256, None, BASE, dict(fluid_substep=1, mg_cycles=2, mg_unfused=1), 4,
     dict(mg_min_size=16, mg_pre=3, mg_post=3)),
    ("512-reference-mg-constants", 512, None, BASE, dict(fluid_substep=1), 3, {}),
    ("384-mg-1+4-3cycles", 384, None, BASE, dict(fluid_substep=1, mg_cycles=3), 3, dict(mg_pre=1, mg_post=4, mg_coarse=7)),
    ("transport-simple-kernel", 128, None, dict(BASE, cohesion=0.7, monomer_pressure=1.0), dict(fluid_substep=1, transport_simple=1),
     4, dict(rubble_frac=0.2)),
    ("long-displacement-rubble", 160, 80, dict(BASE, dt=9.0, cohesion=0.7, monomer_pressure=1.0, aggregation=0.1),
     dict(fluid_substep=1), 4, dict(rubble_frac=0.2, max_disp=2.5, dt=9.0)),
    ("crowded-cells", 96, None, dict(BASE, settle=2.0), dict(fluid_substep=1), 4, dict(monomer_mean=40.0, rubble_frac=0.1)),
    # 200 is not a multiple of the tile sizes: partial tiles at the right and top edges
    ("200-partial-tiles", 200, None, BASE, dict(fluid_substep=1, mg_cycles=2), 3, dict(mg_pre=3, mg_post=3)),
    ("test-cfg-256-128-defaults", 256, 128, dict(dt=1.0), {}, 8, {}),
    ("64-reference-constants", 64, None, dict(BASE, diffusion=30.0, settle=1.0, thermal_activation=1.0,
                                              aggregation=0.02), dict(fluid_substep=1), 10, {}),
    ("jacobi-96", 96, None, BASE, dict(fluid_substep=1, multigrid=0, jacobi_iters=17), 4, {}),
    ("rect-128x64", (128, 64), None, BASE, dict(fluid_substep=1), 6, {}),
    # an odd fluid width: a row pitch that no tensor map can describe, so the
    # stencil tiles are staged with plain loads (one multigrid level)
    ("odd-width-75x48", (150, 96), (75, 48), BASE, dict(fluid_substep=1), 5, {}),
    ("rect-64x128-half-fluid", (64, 128), (32, 64), dict(BASE, monomer_pressure=2.0), dict(fluid_substep=1), 6, {}),
    ("sparse-transport", 64, None, dict(dt=1.0, transport_every=3, aggregation=0.0), dict(fluid_substep=2), 9, {}),
    ("sun-and-vents", 64, None, dict(dt=0.05, sun_heat=1.0, day_period=400.0, activation_decay=0.01,
                                      direct_photoactivation=0.5), dict(fluid_substep=1), 6, {}),
    # the light block (light_mode 1): a sweep on the first step, then propagation / interval sweeps
    ("light-propagate-1-row", 64, None, dict(BASE, direct_photoactivation=0.5), dict(fluid_substep=1, light_mode=1,
                                                                                   light_rows_per_step=1), 6, {}),
    ("light-propagate-3-rows-sun", 96, None, dict(dt=0.05, day_period=300.0, sun_heat=1.0, direct_photoactivation=0.5),
     dict(fluid_substep=1, light_mode=1, light_rows_per_step=3), 6, {}),
    ("light-interval-sweeps", (128, 64), None, dict(BASE, direct_photoactivation=0.5, monomer_uv_absorb=2.0),
     dict(fluid_substep=1, light_mode=1, light_rows_per_step=0, light_interval=2), 6, {}),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_steps_bit_exact(rw, ro, case):
    _, grid, fluid, params, settings, steps, mg = case
    g, o, inputs = setup_pair(rw, ro, grid, fluid, params=params, settings=settings, **mg)
    if case[0] in ("sun-and-vents", "light-propagate-3-rows-sun"):
        rng = np.random.default_rng(3)
        heat = np.zeros(g.field_shape(rw.HEAT)[0], np.float32)
        heat[4:8, 20:24, 0] = 400.0
        heat[4:8, 20:24, 1] = 50.0
        g.upload(rw.HEAT, heat)
        o.upload(rw.HEAT, heat)
        shade = rng.integers(0, 300, size=g.field_shape(rw.SHADE)[0]).astype(np.uint32)
        g.upload(rw.SHADE, shade)
        o.upload(rw.SHADE, shade)
    compare_worlds(g, o, "after upload")
    done = 0
    for batch in (1, 2, steps - 3):
        if batch <= 0:
            continue
        g.encode_steps(batch)
        o.encode_steps(batch)
        done += batch
        compare_worlds(g, o, f"after {done} steps")
    assert g.ledger_blocking() == o.ledger_blocking()


def test_c0_hundred_steps_bit_exact(rw, ro):
    """The c0 configuration in full: 256^2, multigrid 5 levels to 16x16, 2
    V-cycles of 3+3 sweeps, every step a fluid + transport step, 100 steps;
    counts and every field bit-exact with the oracle (checked along the way
    and at the end)."""
    g, o, _ = setup_pair(rw, ro, 256, params=BASE, settings=dict(fluid_substep=1, mg_cycles=2),
                         mg_min_size=16, mg_pre=3, mg_post=3)
    done = 0
    for batch in (50, 50):
        g.encode_steps(batch)
        o.encode_steps(batch)
        done += batch
        compare_worlds(g, o, f"c0 after {done} steps")
    assert done == 100
    assert g.ledger_blocking() == o.ledger_blocking()


def test_graph_replay_matches_direct_launches(rw, ro):
    """Repeated step sequences replay from CUDA graphs; the results must equal
    direct launches and the oracle."""
    import synth

    inputs = synth.make_world_inputs(128, seed=77, rubble_frac=0.1)
    worlds = [rw.World(128, seed=77), rw.World(128, seed=77, no_graphs=1)]
    o = ro.OracleWorld(128, seed=77)
    for w in worlds + [o]:
        w.seed_inputs(inputs)
        for k, v in BASE.items():
            setattr(w.params, k, v)
        w.settings.fluid_substep = 1
    for call in range(6):
        for w in worlds + [o]:
            w.encode_steps(3)
        compare_worlds(worlds[0], o, f"graphs, call {call}")
        compare_worlds(worlds[1], o, f"direct, call {call}")


def test_fluid_disable_clears_once(rw, ro):
    g, o, _ = setup_pair(rw, ro, 64, params=BASE, settings=dict(fluid_substep=1))
    g.encode_steps(2)
    o.encode_steps(2)
    for w in (g, o):
        w.settings.fluid_enabled = 0
    g.encode_steps(3)
    o.encode_steps(3)
    compare_worlds(g, o, "fluid off")
    assert not g.read(rw.VELOCITY).any()


def test_conservation_and_ledger_full_size(rw):
    """2048^2, F = G: ledger after every step equals the seeded counts and
    the CPU recount of the grid (tests/conservation.rs:30-69)."""
    import synth

    n = 2048
    w = rw.World(n, seed=1000, mg_min_size=16, mg_pre=3, mg_post=3)
    w.seed_inputs(synth.make_world_inputs(n, seed=1000))
    w.params = synth.bench_params(1000)
    w.settings.fluid_substep = 1
    w.settings.mg_cycles = 4
    seeded = rw.Ledger.from_cells(w.read_cells_blocking())
    per_channel = [seeded.channel(c) for c in range(4)]
    before = w.read_cells_blocking().copy()
    for _ in range(8):
        w.encode_steps(1)
        led = w.ledger_blocking()
        assert [led.channel(c) for c in range(4)] == per_channel
    cells = w.read_cells_blocking()
    assert rw.Ledger.from_cells(cells) == w.ledger_blocking()
    assert rw.Ledger.from_cells(cells).total() == seeded.total()
    assert (cells != before).mean() > 0.1
    v = w.read(rw.VELOCITY)
    assert np.isfinite(v).all()


def test_deterministic_and_batch_independent(rw):
    """tests/conservation.rs:120-141: bit-identical across runs and across
    64-per-call vs 1-per-call batching."""
    import synth

    def go(batch):
        w = rw.World(256, 128, seed=9)
        w.seed_inputs(synth.make_world_inputs(256, 128, seed=9))
        w.params.dt = 0.5
        done = 0
        while done < 200:
            k = min(batch, 200 - done)
            w.encode_steps(k)
            done += k
        return w.read_cells_blocking(), w.read(rw.VELOCITY)

    a = go(64)
    b = go(64)
    c = go(1)
    assert_same(a[0], b[0], "cells run-to-run")
    assert_same(a[1], b[1], "velocity run-to-run")
    assert_same(a[0], c[0], "cells batched vs single")
    assert_same(a[1], c[1], "velocity batched vs single")


def test_light_sweeps_again_after_a_terrain_upload(rw, ro):
    """Uploading gamma marks the light dirty: the next light block is a full
    sweep on both sides (src/world/mod.rs:1506)."""
    g, o, inputs = setup_pair(rw, ro, 64, params=dict(BASE, direct_photoactivation=0.5),
                              settings=dict(fluid_substep=1, light_mode=1, light_rows_per_step=1))
    g.encode_steps(3)
    o.encode_steps(3)
    gamma = inputs[rw.GAMMA].copy()
    gamma[20:30, 10:50] = 6
    g.upload(rw.GAMMA, gamma)
    o.upload(rw.GAMMA, gamma)
    g.encode_steps(3)
    o.encode_steps(3)
    compare_worlds(g, o, "after the terrain upload")
    assert_same(g.read(rw.LIGHT), o.read(rw.LIGHT), "light")


def test_async_ledger_readback(rw):
    """encode_ledger_readback / poll_ledger: the ledger of the state when it
    was requested, delivered without waiting, one readback at a time."""
    import time

    import synth

    w = rw.World(128, seed=12)
    w.seed_inputs(synth.make_world_inputs(128, seed=12))
    w.params.dt = 1.0
    w.settings.fluid_substep = 1
    w.encode_steps(3)
    assert w.poll_ledger() is None                      # nothing requested
    want = rw.Ledger.from_cells(w.read_cells_blocking())
    w.request_ledger()
    w.request_ledger()                                  # pending: does nothing
    w.encode_steps(4)                                   # recorded after the request
    got, t_end = None, time.time() + 30.0
    while got is None and time.time() < t_end:
        got = w.poll_ledger()
    assert got == want
    assert w.poll_ledger() is None                      # the readback is over
    w.sync()
    w.request_ledger()
    w.sync()
    assert w.poll_ledger() == w.ledger_blocking()


def _bench_pair(rw, ro, n, seed=1000, mg_cluster=0):
    """A GPU world and an oracle world with the benchmark's settings: F = G,
    multigrid to 16x16, 4 V-cycles of 3+3 sweeps, 30 coarse sweeps, fluid and
    transport every step, dt = 1, sun heating off, reference defaults (the
    oracle's own table on its side)."""
    import synth

    g = rw.World(n, seed=seed, mg_min_size=16, mg_pre=3, mg_post=3, mg_cluster=mg_cluster)
    o = ro.OracleWorld(n, seed=seed, mg_min_size=16, mg_pre=3, mg_post=3)
    inputs = synth.make_world_inputs(n, seed=seed)
    g.seed_inputs(inputs)
    o.seed_inputs(inputs)
    g.params = synth.bench_params(seed)
    o.params = synth.bench_params(seed, defaults=ro.default_params)
    assert bytes(g.params) == bytes(o.params), "the library's default table differs from the oracle's"
    for w in (g, o):
        w.settings.fluid_substep = 1
        w.settings.mg_cycles = 4
    return g, o


@pytest.mark.parametrize("n,steps", [(2048, 2), (1024, 3)], ids=["2048-bench-config", "1024-big-box-multigrid"])
def test_benchmark_configuration_bit_exact(rw, ro, n, steps):
    """The configuration the benchmark times, stepped on the GPU and on the
    oracle, every field compared bit for bit after each step.  At 2048^2 and
    1024^2 the two finest multigrid levels run the 66 x 50 box kernels (the
    level picks them once it has three tiles per SM), which smaller parity
    cases never reach; 2048^2 is the benchmark's own size and schedule
    (src/world/mod.rs:1545-1577 with MG_PRE = MG_POST = 3, 4 cycles, 8
    levels)."""
    g, o = _bench_pair(rw, ro, n)
    compare_worlds(g, o, f"{n}^2 after upload")
    for s in range(steps):
        g.encode_steps(1)
        o.encode_steps(1)
        compare_worlds(g, o, f"{n}^2 after {s + 1} steps")
    assert g.ledger_blocking() == o.ledger_blocking()
    g.close()
    o.close()


@pytest.mark.parametrize("cluster", [8, 1], ids=["cluster-8", "no-cluster"])
@pytest.mark.parametrize("n,steps", [(256, 4), (2048, 1)], ids=["256", "2048"])
def test_multigrid_cluster_choices_bit_exact(rw, ro, n, steps, cluster):
    """The small multigrid levels on an 8-CTA cluster (at 256^2 that changes
    which levels are slabs: 64^2 and 32^2 only) and without a cluster (a box
    launch per level and the single-CTA coarse kernel), against the oracle:
    every way of running the V-cycle gives the reference's bits."""
    g, o = _bench_pair(rw, ro, n, mg_cluster=cluster)
    for s in range(steps):
        g.encode_steps(1)
        o.encode_steps(1)
        compare_worlds(g, o, f"{n}^2 mg_cluster={cluster} after {s + 1} steps")
    g.close()
    o.close()
