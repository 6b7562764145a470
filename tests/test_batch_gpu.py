"""Batched stepping through the C ABI: every member of a batch -- worlds of
different sizes, shapes and settings -- gets exactly the bits it gets when
stepped alone, and small members match the oracle."""
import numpy as np
import pytest

import synth
from helpers import STATE_FIELDS, assert_same, compare_worlds

pytestmark = pytest.mark.gpu

BASE = dict(dt=1.0, transport_every=1, sun_heat=0.0, day_period=0.0)
MG33 = dict(mg_min_size=16, mg_pre=3, mg_post=3)
FULL = dict(fluid_substep=1, mg_cycles=2)

# grid, fluid, params, settings, world kwargs, synth kwargs
MIXED = [
    (128, None, BASE, FULL, MG33, {}),
    (192, None, BASE, FULL, MG33, dict(rock_frac=0.2, monomer_mean=7.0)),
    ((256, 64), None, BASE, FULL, MG33, dict(rock_frac=0.05)),
    ((64, 128), (32, 64), dict(BASE, monomer_pressure=2.0), FULL, MG33, {}),
    (96, None, dict(BASE, aggregation=0.05, cohesion=0.6), FULL, MG33, dict(rubble_frac=0.1)),
    # reference multigrid constants: a group of its own
    (128, None, BASE, dict(fluid_substep=1), {}, {}),
    # fluid every second step: joins the other groups on even epochs only
    (64, None, BASE, dict(fluid_substep=2, mg_cycles=2), MG33, {}),
    # one dispatch per half-sweep, and Jacobi: per-world pressure solves inside the batch
    (80, None, BASE, dict(FULL, mg_unfused=1), MG33, {}),
    (64, None, BASE, dict(fluid_substep=1, multigrid=0, jacobi_iters=10), {}, {}),
]


def make_world(rw, spec, seed):
    grid, fluid, params, settings, wkw, skw = spec
    w = rw.World(grid, fluid, seed=seed, **wkw)
    w.seed_inputs(synth.make_world_inputs(grid, fluid, seed=seed, **skw))
    for k, v in params.items():
        setattr(w.params, k, v)
    for k, v in settings.items():
        setattr(w.settings, k, v)
    return w


def twins(rw, specs, ledgers=False):
    batch_worlds, alone = [], []
    for i, spec in enumerate(specs):
        for lst in (batch_worlds, alone):
            w = make_world(rw, spec, 1000 + i)
            w.settings.ledger_each_step = 1 if ledgers else 0
            lst.append(w)
    return batch_worlds, alone


def compare_all(a_list, b_list, what):
    for k, (a, b) in enumerate(zip(a_list, b_list)):
        for f, name in STATE_FIELDS:
            assert_same(a.read(f), b.read(f), f"{what}: member {k}: {name}")


def test_mixed_batch_equals_alone(rw):
    members, alone = twins(rw, MIXED)
    b = rw.Batch(members)
    # 4-step calls repeat their graph key from the third one on: first run
    # direct, then captured, then replayed
    for n in (1, 2, 4, 4, 4, 3):
        b.encode_steps(n)
        for w in alone:
            w.encode_steps(n)
        b.sync()
        compare_all(members, alone, f"after a {n}-step call")
    assert [w.params.epoch for w in members] == [w.params.epoch for w in alone]
    b.close()


def test_mixed_precision_members_equal_alone(rw):
    # Members that solve every step's pressure to the mixed-precision
    # tolerance share the batch's launches with f32 members (their solves run
    # one world at a time) and get the bits they get alone: pressure pair,
    # velocity, transport.
    specs = [(128, None, BASE, FULL, dict(MG33, precision_mode=1), {}),
             ((256, 128), None, BASE, FULL, dict(MG33, precision_mode=1), dict(rock_frac=0.2)),
             MIXED[0], MIXED[2]]
    members, alone = twins(rw, specs)
    b = rw.Batch(members)
    for n in (1, 2, 2, 2):
        b.encode_steps(n)
        for w in alone:
            w.encode_steps(n)
        b.sync()
        for k, (a, w) in enumerate(zip(members, alone)):
            fields = STATE_FIELDS + ([(rw.PRESSURE_LO, "pressure_lo")] if k < 2 else [])
            for f, name in fields:
                assert_same(a.read(f), w.read(f), f"after a {n}-step call: member {k}: {name}")
    for k in (0, 1):
        outer, inner, rho = members[k].solve_info()
        assert rho <= 1e-5, (k, outer, inner, rho)
    b.close()


def test_batch_members_match_oracle(rw, ro):
    specs = [MIXED[3], MIXED[4], MIXED[6]]
    members = [make_world(rw, s, 77 + i) for i, s in enumerate(specs)]
    oracles = []
    for i, (grid, fluid, params, settings, wkw, skw) in enumerate(specs):
        o = ro.OracleWorld(grid, fluid, seed=77 + i, **wkw)
        o.seed_inputs(synth.make_world_inputs(grid, fluid, seed=77 + i, **skw))
        for k, v in params.items():
            setattr(o.params, k, v)
        for k, v in settings.items():
            setattr(o.settings, k, v)
        oracles.append(o)
    b = rw.Batch(members)
    for n in (1, 3):
        b.encode_steps(n)
        for o in oracles:
            o.encode_steps(n)
        b.sync()
        for k, (g, o) in enumerate(zip(members, oracles)):
            compare_worlds(g, o, f"member {k} after {n} steps")
    b.close()


def test_batch_step_ledgers_equal_alone(rw):
    members, alone = twins(rw, MIXED[:5] + MIXED[6:7], ledgers=True)
    b = rw.Batch(members)
    b.encode_steps(5)
    for w in alone:
        w.encode_steps(5)
    got = b.step_ledgers(5)
    for k, w in enumerate(alone):
        want = w.step_ledgers(5)
        for i in range(5):
            assert got[k][i] == want[i], (k, i)
        # conservation: transport moves and reacts monomers, never creates them
        first = got[k][0]
        for led in got[k]:
            assert led.total() == first.total()
    b.close()


@pytest.mark.parametrize("modes", [[1, 1, 1, 1, 1], [2, 2, 2, 2, 2], [1, 2, 1, 2, 1]])
def test_tile_shapes_do_not_change_results(rw, modes):
    specs = [(512, None, BASE, FULL, MG33, {}), ((1024, 128), None, BASE, FULL, MG33, {}), MIXED[0], MIXED[2]]
    members, alone = twins(rw, specs)
    b = rw.Batch(members)
    b.set_tile_modes(modes)
    b.encode_steps(3)
    for w in alone:
        w.encode_steps(3)
    b.sync()
    compare_all(members, alone, f"tile modes {modes}")
    b.close()


def test_autotune_then_step(rw):
    members, alone = twins(rw, MIXED[:4])
    b = rw.Batch(members)
    modes = b.autotune()
    assert all(m in (0, 1, 2) for m in modes)
    b.encode_steps(4)
    for w in alone:
        w.encode_steps(4)
    b.sync()
    compare_all(members, alone, f"after autotune {modes}")
    b.close()


def test_membership_changes(rw):
    members, alone = twins(rw, MIXED[:4])
    b = rw.Batch(members[:3])
    b.encode_steps(2)
    for w in alone[:3]:
        w.encode_steps(2)
    # a world joins late, another leaves and keeps stepping on its own
    b.add(members[3])
    alone[3].encode_steps(0)
    b.remove(members[0])
    b.encode_steps(3)
    for w in alone[1:]:
        w.encode_steps(3)
    members[0].encode_steps(3)
    alone[0].encode_steps(3)
    b.sync()
    compare_all(members, alone, "after membership changes")
    b.close()
    # the released worlds step on their own streams again
    members[1].encode_steps(1)
    alone[1].encode_steps(1)
    compare_all(members[1:2], alone[1:2], "after the batch closed")


def test_batch_rejects_bad_arguments(rw):
    w = make_world(rw, MIXED[0], 5)
    b1 = rw.Batch([w])
    b2 = rw.Batch()
    with pytest.raises(rw.RiboError):
        b2.add(w)  # already a member of b1
    with pytest.raises(rw.RiboError):
        b2.remove(w)  # not a member
    with pytest.raises(rw.RiboError):
        b1.set_tile_modes([3])
    b1.close()
    b2.add(w)
    b2.close()


def test_batches_reject_the_light_block(rw):
    import synth

    w = rw.World(64, seed=4)
    w.seed_inputs(synth.make_world_inputs(64, seed=4))
    w.settings.light_mode = 1
    b = rw.Batch()
    b.add(w)
    w._sync_settings()
    with pytest.raises(rw.RiboError, match="frozen input"):
        b.encode_steps(1)
