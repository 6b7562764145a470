"""CPU checks of the oracle: pinned math accuracy, an independent restatement
of the PCG4D hash, and the reference's own world invariants
(tests/conservation.rs) run on the oracle."""
import math

import numpy as np
import pytest

import ribo_world as rw


def ulp_err(got: float, exact: float) -> float:
    g = np.float32(got)
    e = np.float64(exact)
    if not np.isfinite(e):
        return 0.0 if g == e else np.inf
    spacing = np.spacing(np.float32(abs(e))) if e != 0 else np.float32(1e-45)
    return float(abs(np.float64(g) - e) / np.float64(spacing))


def test_pinned_exp_accuracy(ro):
    lib = ro.load()
    xs = np.concatenate([np.linspace(-87, 88, 20001), np.linspace(-1, 1, 5001), np.array([0.0, -0.0, 1e-8, -1e-8])])
    worst = 0.0
    for x in xs.astype(np.float32):
        worst = max(worst, ulp_err(lib.orc_exp(float(x)), math.exp(float(x))))
    assert worst <= 2.0, worst
    assert lib.orc_exp(-200.0) == 0.0
    assert math.isinf(lib.orc_exp(100.0))
    assert lib.orc_exp(0.0) == 1.0


def test_pinned_log_pow_sin_accuracy(ro):
    lib = ro.load()
    worst_log = max(ulp_err(lib.orc_log(float(x)), math.log(float(x)))
                    for x in np.geomspace(1e-30, 1e30, 20001).astype(np.float32) if abs(math.log(float(x))) > 1e-3)
    assert worst_log <= 3.0, worst_log
    # pow = exp(y * ln x) in f32: the error grows with |y ln x|.  The world
    # step calls it as pow(fluid_decay, 60 * fluid_dt) with |y ln x| < 1.
    worst_pow, worst_rel = 0.0, 0.0
    for x in np.linspace(0.01, 1.0, 200).astype(np.float32):
        for y in np.linspace(0.0, 10.0, 41).astype(np.float32):
            exact = float(x) ** float(y)
            got = lib.orc_pow(float(x), float(y))
            if abs(float(y) * math.log(float(x))) <= 1.0:
                worst_pow = max(worst_pow, ulp_err(got, exact))
            worst_rel = max(worst_rel, abs(got - exact) / exact)
    assert worst_pow <= 4.0, worst_pow
    assert worst_rel <= 1e-5, worst_rel
    assert lib.orc_pow(0.0, 4.2) == 0.0 and lib.orc_pow(1.0, 3.0) == 1.0 and lib.orc_pow(0.5, 0.0) == 1.0
    worst_sin = 0.0
    for x in np.linspace(-20.0, 20.0, 40001).astype(np.float32):
        s = math.sin(float(x))
        if abs(s) > 1e-3:
            worst_sin = max(worst_sin, ulp_err(lib.orc_sin(float(x)), s))
    assert worst_sin <= 4.0, worst_sin


def pcg4d_numpy(v):
    """shaders/common/rng.wgsl:10-23, restated with numpy uint32 arithmetic."""
    v = [np.uint32(x) for x in v]
    with np.errstate(over="ignore"):
        v = [x * np.uint32(1664525) + np.uint32(1013904223) for x in v]
        x, y, z, w = v
        x = x + y * w
        y = y + z * x
        z = z + x * y
        w = w + y * z
        x, y, z, w = [t ^ (t >> np.uint32(16)) for t in (x, y, z, w)]
        x = x + y * w
        y = y + z * x
        z = z + x * y
        w = w + y * z
    return [int(x), int(y), int(z), int(w)]


def test_pcg4d_matches_independent_restatement(ro):
    import ctypes

    lib = ro.load()
    rng = np.random.default_rng(0)
    out = (ctypes.c_uint32 * 4)()
    for _ in range(2000):
        a = [int(t) for t in rng.integers(0, 2**32, size=4, dtype=np.uint64)]
        lib.orc_pcg4d(*a, out)
        assert list(out) == pcg4d_numpy(a)
    # rng_f4 uses the top 24 bits: (u >> 8) / 2^24 is exact in f32
    lib.orc_pcg4d(0, 0, 0, 1, out)
    assert list(out) == pcg4d_numpy([0, 0, 0, 1])


def _vent_world(ro, n, fluid=None, seed=7, **params):
    import synth

    o = ro.OracleWorld(n, fluid, seed=seed)
    inp = synth.make_world_inputs(n, fluid, seed=seed)
    o.seed_inputs(inp)
    fw = n if fluid is None else fluid
    heat = np.zeros((fw, fw, 2), np.float32)
    c = fw // 2
    heat[1:3, c - 2:c + 2, 0] = 3000.0  # a vent at the bottom centre (x = heat, y = reductant)
    heat[1:3, c - 2:c + 2, 1] = 100.0
    o.upload(rw.HEAT, heat)
    for k, v in params.items():
        setattr(o.params, k, v)
    return o, inp


def test_oracle_matter_is_conserved_exactly(ro):
    """tests/conservation.rs:30-69 on the oracle (128^2 world, 64^2 fluid)."""
    o, inp = _vent_world(ro, 128, 64, diffusion=30.0, settle=1.0, thermal_activation=1.0, aggregation=0.02)
    seeded = rw.Ledger.from_cells(inp[rw.CHEM])
    assert seeded.total() > 0
    assert o.ledger_blocking() == seeded
    o.run(640)
    cells = o.read_cells_blocking()
    after = rw.Ledger.from_cells(cells)
    moved = int((cells != inp[rw.CHEM].reshape(-1)).sum())
    assert moved > cells.size // 10
    assert sum(after.act) != sum(seeded.act), "no reaction changed the state"
    assert after.total() == seeded.total()
    assert [after.channel(c) for c in range(4)] == [seeded.channel(c) for c in range(4)]
    assert o.ledger_blocking() == after


def test_oracle_fluid_is_sane(ro):
    """tests/conservation.rs:72-115 (fluid part): the vent heats the water and
    sets it moving, everything stays finite, and the net vertical flux through
    rows n/4, n/2, 3n/4 is below 10 % of the gross flux."""
    o, _ = _vent_world(ro, 64, seed=3, day_period=0.0, uv_depth=2.0)
    o.upload(rw.VELOCITY, np.zeros((64, 64, 2), np.float32))
    o.run(600)
    vel = o.read(rw.VELOCITY)
    temp = o.read(rw.TEMP)
    assert np.isfinite(vel).all() and np.isfinite(temp).all()
    assert temp.max() > 2.0
    speed = np.sqrt((vel.astype(np.float64) ** 2).sum(-1))
    assert speed.max() > 0.1
    n = 64
    for y in (n // 4, n // 2, 3 * n // 4):
        net = vel[y, :, 1].sum()
        gross = np.abs(vel[y, :, 1]).sum()
        assert abs(net) < 0.1 * max(gross, n), (y, net, gross)


def test_oracle_is_deterministic_and_batch_independent(ro):
    """tests/conservation.rs:120-141: bit-identical across runs, across 64-
    vs 1-step batching and across OpenMP thread counts."""
    import synth

    def go(batch, threads):
        ro.set_threads(threads)
        o = ro.OracleWorld(64, 32, seed=9)
        o.seed_inputs(synth.make_world_inputs(64, 32, seed=9))
        o.params.dt = 0.5
        done = 0
        while done < 96:
            k = min(batch, 96 - done)
            o.encode_steps(k)
            done += k
        return o.read_cells_blocking(), o.read(rw.VELOCITY)

    import os

    nt = os.cpu_count() or 2
    a = go(64, nt)
    b = go(64, nt)
    c = go(1, 1)
    ro.set_threads(nt)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    assert np.array_equal(a[0], c[0]) and np.array_equal(a[1].view(np.uint32), c[1].view(np.uint32))


def test_oracle_sparse_transport_conserves_matter(ro):
    """tests/conservation.rs:274-292: transport every 3 steps."""
    o, inp = _vent_world(ro, 96, 48, seed=5, diffusion=10.0, settle=1.0, thermal_activation=1.0,
                         aggregation=0.02, transport_every=3)
    seeded = rw.Ledger.from_cells(inp[rw.CHEM])
    o.run(300)
    cells = o.read_cells_blocking()
    after = rw.Ledger.from_cells(cells)
    assert int((cells != inp[rw.CHEM].reshape(-1)).sum()) > cells.size // 10
    assert after.total() == seeded.total()
    assert [after.channel(c) for c in range(4)] == [seeded.channel(c) for c in range(4)]


@pytest.mark.parametrize("n,levels", [(2048, 8), (256, 6), (128, 5), (96, 5), (100, 3), (8, 1)])
def test_multigrid_level_rule(ro, n, levels):
    """src/world/mod.rs:637-641: halve while above MG_MIN_SIZE and even
    (2048 with MG_MIN_SIZE 16 gives the 8 levels of the benchmark)."""
    o = ro.OracleWorld(n if n <= 256 else 32, seed=1, mg_min_size=16 if n == 2048 else 8)
    if n <= 256:
        assert o.num_levels() == levels
    else:
        sizes = [n]
        while sizes[-1] > 16 and sizes[-1] % 2 == 0:
            sizes.append(sizes[-1] // 2)
        assert len(sizes) == levels


def test_oracle_default_settings_match_the_library(rw, ro):
    """Both sides start from the reference's WorldSettings defaults
    (src/world/mod.rs:117-134), so a test that sets only some fields compares
    like with like (the mixed-solver fields, which the oracle does not run,
    take their defaults from zero)."""
    import ctypes

    lib = rw.load_library()
    want = rw.WorldSettings()
    lib.ribo_world_settings_default(ctypes.byref(want))
    got = ro._default_settings()
    for name, _ in rw.WorldSettings._fields_:
        if name.startswith("mixed_"):
            continue
        assert getattr(got, name) == getattr(want, name), name
