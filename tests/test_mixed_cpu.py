"""The FP64 pressure oracle (oracle/fp64_pressure.py) is the operator the
reference's multigrid solves: its FP64 solution is a fixed point of the
oracle's f32 V-cycles (a restatement of shaders/world/multigrid.wgsl)."""
import numpy as np
import pytest

import fp64_pressure as fp
import synth


def world_after_steps(ro, rw, n, steps=2, seed=7):
    o = ro.OracleWorld(n, seed=seed, mg_min_size=8, mg_pre=2, mg_post=2, mg_coarse=30)
    o.seed_inputs(synth.make_world_inputs(n, seed=seed))
    bp = synth.bench_params(seed)
    for k, _ in rw.SimParams._fields_:
        setattr(o.params, k, getattr(bp, k))
    o.settings.fluid_substep = 1
    o.encode_steps(steps)
    return o


def test_operator_matrix_matches_apply(ro, rw):
    o = world_after_steps(ro, rw, 48)
    water = o.read(rw.SOLID_MASK) == 0
    A, cells = fp.operator(water)
    p = np.random.default_rng(1).standard_normal(water.shape)
    p = np.where(water, p, 0.0)
    assert np.allclose((A @ p.reshape(-1)[cells]), fp.apply(p, water).reshape(-1)[cells], rtol=0, atol=1e-12)
    # symmetric, and the constant vector of a water region is an eigenvector (eigenvalue -eps0)
    assert abs(A - A.T).max() == 0
    assert np.allclose(fp.apply(np.ones(water.shape), water)[water], -fp.EPS0, rtol=0, atol=1e-15)


def test_fp64_solve_residual(ro, rw):
    o = world_after_steps(ro, rw, 64)
    water = o.read(rw.SOLID_MASK) == 0
    rhs = o.read(rw.DIVERGENCE)
    p = fp.solve(rhs, water)
    assert fp.rel_residual(p, rhs, water) < 1e-10


def test_fp64_solution_is_a_fixed_point_of_the_reference_multigrid(ro, rw):
    o = world_after_steps(ro, rw, 64)
    water = o.read(rw.SOLID_MASK) == 0
    rhs = o.read(rw.DIVERGENCE)
    want = fp.solve(rhs, water)
    # warm-start the reference's f32 V-cycles at the FP64 solution: they must
    # leave it where it is (up to FP32 rounding), as they do any solution of
    # the operator they smooth
    o.upload(rw.PRESSURE, want.astype(np.float32))
    o.settings.mg_cycles = 4
    o.run_pass(o.params, 8)
    got = o.read(rw.PRESSURE).astype(np.float64)
    moved = np.linalg.norm(np.where(water, got - want, 0)) / np.linalg.norm(want)
    assert moved < 1e-5, moved
    # while from zero the same V-cycles are far from it (the check has teeth)
    o.upload(rw.PRESSURE, np.zeros_like(want, np.float32))
    o.run_pass(o.params, 8)
    far = o.read(rw.PRESSURE).astype(np.float64)
    assert np.linalg.norm(np.where(water, far - want, 0)) / np.linalg.norm(want) > 1e-2


def test_benchmark_residual_matches_the_fp64_oracle():
    """bench.py re-checks the mixed-precision solve with its own FP64 residual
    (it may not call the oracle); both evaluate ||rhs - L p|| / ||rhs|| with the
    same level-0 operator."""
    import os
    import sys

    import numpy as np

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    import fp64_pressure as fp

    rng = np.random.default_rng(5)
    for shape in ((33, 47), (64, 64)):
        water = rng.random(shape) > 0.15
        p = rng.standard_normal(shape) * 3.0
        b = rng.standard_normal(shape)
        assert bench.host_rel_residual(p, b, water) == fp.rel_residual(p, b, water)
