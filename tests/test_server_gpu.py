"""Serving with continuous batching: jobs that arrive while others run, are
admitted as memory frees up and share launches with them, finish with
exactly the bits the same job gets when its world is stepped alone."""
import numpy as np
import pytest

import synth
from helpers import assert_same

pytestmark = pytest.mark.gpu

def job_specs():
    # grid, steps, synth kwargs, settings
    return [
        ((128, 128), 13, dict(rock_frac=0.1), dict(fluid_substep=1, mg_cycles=2)),
        ((256, 64), 40, dict(rock_frac=0.2, monomer_mean=6.0), dict(fluid_substep=1, mg_cycles=2)),
        ((192, 192), 7, dict(rock_frac=0.05), dict(fluid_substep=1, mg_cycles=2)),
        ((64, 256), 25, dict(rock_frac=0.15, monomer_mean=2.0), dict(fluid_substep=2, mg_cycles=1)),
        ((320, 160), 18, dict(rock_frac=0.1), dict(fluid_substep=1, mg_cycles=2)),
        ((128, 128), 33, dict(rock_frac=0.25, monomer_mean=8.0), dict(fluid_substep=1, mg_cycles=2, ledger_each_step=1)),
        ((96, 96), 5, dict(rock_frac=0.1), dict(fluid_substep=1, mg_cycles=2)),
    ]


def make_job(rw, i, spec):
    grid, steps, skw, settings = spec
    inputs = synth.make_world_inputs(grid, seed=3000 + i, **skw)
    params = synth.bench_params(3000 + i)
    st = rw.default_settings()
    for k, v in settings.items():
        setattr(st, k, v)
    return grid, steps, inputs, params, st


def run_alone(rw, grid, steps, inputs, params, st):
    w = rw.World(grid, seed=1, mg_min_size=16, mg_pre=3, mg_post=3)
    w.seed_inputs(inputs)
    w.params = params.copy()
    w.settings = st
    w.run(steps)
    out = {f: w.read(f) for f in (rw.CHEM, rw.VELOCITY, rw.PRESSURE, rw.TEMP, rw.DIVERGENCE)}
    led = w.ledger_blocking()
    w.close()
    return out, led


def test_served_jobs_equal_alone(rw):
    fields = (rw.CHEM, rw.VELOCITY, rw.PRESSURE, rw.TEMP, rw.DIVERGENCE)
    jobs = [make_job(rw, i, s) for i, s in enumerate(job_specs())]
    # the budget holds about three of these worlds at a time, so later jobs queue
    fps = [rw.world_footprint(j[0], mg_min_size=16) for j in jobs]
    budget = int(sorted(fps)[-1] + sorted(fps)[-2] + sorted(fps)[-3])
    srv = rw.Server(budget, max_chunk_steps=8)
    ids = {}
    arrivals = [0, 0, 0, 1, 2, 2, 4]  # iteration before which each job arrives
    it = 0
    pending = list(range(len(jobs)))
    max_active = 0
    while pending or srv.stats().active or srv.stats().pending:
        for i in list(pending):
            if arrivals[i] <= it:
                grid, steps, inputs, params, st = jobs[i]
                ids[srv.submit(grid, steps=steps, params=params, settings=st, inputs=inputs, outputs=fields,
                               mg_min_size=16, mg_pre=3, mg_post=3, user_tag=i)] = i
                pending.remove(i)
        max_active = max(max_active, srv.iterate())
        assert srv.stats().bytes_in_use <= budget
        it += 1
        assert it < 1000
    srv.drain()
    results = srv.results()
    assert len(results) == len(jobs)
    assert max_active >= 2  # jobs really shared the GPU
    for r, outs in results:
        i = r.user_tag
        assert r.status == 0
        grid, steps, inputs, params, st = jobs[i]
        assert r.steps == steps
        assert r.t_submit_ms <= r.t_admit_ms <= r.t_done_ms
        want, led = run_alone(rw, grid, steps, inputs, params, st)
        for f in fields:
            assert_same(outs[f], want[f], f"job {i} field {f}")
        assert list(r.ledger) == [led.act[c] for c in range(4)] + [led.spent[c] for c in range(4)] + [0, 0, 0, 0]
    its = srv.iterations()
    assert its and all(ms > 0 and steps >= 1 for ms, steps, _ in its)
    s = srv.stats()
    assert s.completed == len(jobs) and s.active == 0 and s.pending == 0 and s.bytes_in_use == 0
    assert s.world_steps == sum(j[1] for j in jobs)
    srv.close()


def test_served_mixed_precision_jobs_equal_alone(rw):
    # jobs that solve each pressure to the mixed-precision tolerance, served
    # side by side with an f32 job, finish with the bits they get alone
    base = (rw.CHEM, rw.VELOCITY, rw.PRESSURE, rw.DIVERGENCE)
    specs = [((128, 128), 9, 1), ((192, 96), 6, 1), ((128, 128), 7, 0)]
    srv = rw.Server(1 << 34, max_chunk_steps=4)
    jobs = {}
    for i, (grid, steps, mode) in enumerate(specs):
        inputs = synth.make_world_inputs(grid, seed=4000 + i)
        params = synth.bench_params(4000 + i)
        st = rw.default_settings()
        st.fluid_substep = 1
        st.mg_cycles = 2
        fields = base + ((rw.PRESSURE_LO,) if mode else ())
        jid = srv.submit(grid, steps=steps, params=params, settings=st, inputs=inputs, outputs=fields,
                         mg_min_size=16, mg_pre=3, mg_post=3, user_tag=i, precision_mode=mode)
        jobs[i] = (grid, steps, mode, inputs, params, st, fields)
    srv.drain()
    results = srv.results()
    assert len(results) == len(specs)
    for r, outs in results:
        assert r.status == 0
        grid, steps, mode, inputs, params, st, fields = jobs[r.user_tag]
        w = rw.World(grid, seed=1, mg_min_size=16, mg_pre=3, mg_post=3, precision_mode=mode)
        w.seed_inputs(inputs)
        w.params = params.copy()
        w.settings = st
        w.run(steps)
        for f in fields:
            assert_same(outs[f], w.read(f), f"job {r.user_tag} field {f}")
        w.close()
    srv.close()


def test_over_budget_job_is_refused(rw):
    srv = rw.Server(10 * 1024 * 1024, max_chunk_steps=4)
    with pytest.raises(rw.RiboError) as e:
        srv.submit(512, steps=3, params=synth.bench_params(1))
    assert "OVER_BUDGET" in str(e.value)
    srv.close()


def test_world_memory_equals_footprint(rw):
    import ctypes

    lib = rw.load_library()
    for grid, mg in (((128, 64), 8), ((256, 256), 16), ((96, 192), 8)):
        w = rw.World(grid, mg_min_size=mg)
        got = ctypes.c_uint64()
        assert lib.ribo_world_memory(w._h, ctypes.byref(got)) == 0
        assert got.value == rw.world_footprint(grid, mg_min_size=mg)
        w.close()
