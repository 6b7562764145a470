"""Mixed-precision pressure solve on the GPU: every solve reaches the relative
residual tolerance against the FP64 operator (checked on the host in FP64
from the pressure pair the GPU left), its solution agrees with the FP64
oracle solve, and transport stays bit-exact with the oracle."""
import numpy as np
import pytest

import fp64_pressure as fp
import synth
from helpers import assert_same

pytestmark = pytest.mark.gpu

MIXED = 1
TOL = 1e-5


def mixed_world(rw, grid, seed=11, no_graphs=0, **skw):
    w = rw.World(grid, seed=seed, mg_min_size=16, mg_pre=3, mg_post=3, precision_mode=MIXED, no_graphs=no_graphs)
    w.seed_inputs(synth.make_world_inputs(grid, seed=seed, **skw))
    w.params = synth.bench_params(seed)
    w.settings.fluid_substep = 1
    return w


def check_solve(rw, w, what):
    water = w.read(rw.SOLID_MASK) == 0
    rhs = w.read(rw.DIVERGENCE)
    p = w.read(rw.PRESSURE).astype(np.float64) + w.read(rw.PRESSURE_LO).astype(np.float64)
    rho = fp.rel_residual(p, rhs, water)
    outer, inner, rho_dev = w.solve_info()
    assert rho <= TOL, f"{what}: host FP64 relative residual {rho:.3e} (device {rho_dev:.3e}, {outer} outer, {inner} CG)"
    assert abs(rho - rho_dev) <= 1e-2 * TOL + 1e-3 * rho, (what, rho, rho_dev)
    return p, water, rhs, (outer, inner, rho)


@pytest.mark.parametrize("grid", [256, (512, 256)])
def test_each_solve_reaches_tolerance(rw, grid):
    w = mixed_world(rw, grid)
    for call in range(4):
        w.encode_steps(1)
        p, water, rhs, info = check_solve(rw, w, f"step {call + 1}")
        if call == 0:
            want = fp.solve(rhs, water)
            err = np.linalg.norm(np.where(water, p - want, 0)) / np.linalg.norm(want)
            assert err < 1e-3, err
    w.close()


def test_graph_replay_and_direct_agree(rw):
    # the step graph embeds the solve's device-side loops; without graphs the
    # solve runs as its own graph: both reach the tolerance
    a = mixed_world(rw, 256)
    b = mixed_world(rw, 256, no_graphs=1)
    for n in (2, 2, 2, 2):
        a.encode_steps(n)
        b.encode_steps(n)
    pa = check_solve(rw, a, "graphs")[0]
    pb = check_solve(rw, b, "direct")[0]
    assert np.linalg.norm(pa - pb) <= 1e-3 * np.linalg.norm(pb)
    a.close()
    b.close()


def test_transport_is_bit_exact_in_mixed_mode(rw, ro):
    w = mixed_world(rw, 256, seed=5)
    w.encode_steps(2)
    chem0 = w.read(rw.CHEM)
    gamma = w.read(rw.GAMMA)
    step = w.params.copy()
    w.encode_steps(1)
    # the transport block of that step, on the oracle, from the GPU's state:
    # the chem before the step and the velocity the fluid block left
    o = ro.OracleWorld(256, seed=5, mg_min_size=16, mg_pre=3, mg_post=3)
    o.upload(rw.GAMMA, gamma)
    o.upload(rw.CHEM, chem0)
    o.upload(rw.LIGHT, w.read(rw.LIGHT))
    o.upload(rw.VELOCITY, w.read(rw.VELOCITY))
    o.upload(rw.TEMP, w.read(rw.TEMP))
    o.settings.fluid_substep = 1
    params = rw.derive_step_params(step, w.settings, 1)[0]
    o.run_pass(params, 13)  # thermal activation
    if params.aggregation > 0:
        o.run_pass(params, 14)
    o.run_pass(params, 15)  # transport scatter + commit
    assert_same(w.read(rw.CHEM), o.read(rw.CHEM), "chem after the mixed-mode step")
    w.close()


def test_mixed_mode_rejections(rw):
    with pytest.raises(rw.RiboError):
        rw.World(64, mg_min_size=16, precision_mode=MIXED)  # everything fits the coarse kernel
    with pytest.raises(rw.RiboError):
        rw.World((2048, 256), mg_min_size=16, precision_mode=MIXED)  # coarsest level 128x16, above 1024 cells
    w = mixed_world(rw, 256)
    f = rw.World(128)
    with pytest.raises(rw.RiboError):
        f.solve_info()
    with pytest.raises(rw.RiboError):
        f.read(rw.PRESSURE_LO)
    f.close()
    w.close()


def test_full_size_solves_reach_tolerance(rw):
    """The mixed-precision configuration at the benchmark's size (2048^2,
    FP16-storage levels 0-3, FP32 defect correction, FP64 coarsest solve and
    mean removal): each of two steps' solves reaches a relative residual of
    1e-5 against the FP64 operator, evaluated on the host in FP64 from the
    pressure pair the GPU left."""
    w = mixed_world(rw, 2048, seed=1000)
    for call in range(2):
        w.encode_steps(1)
        check_solve(rw, w, f"2048^2 step {call + 1}")
    w.close()
