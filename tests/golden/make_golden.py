"""Generates the golden fixtures of the world step with the CPU oracle.

Each fixture holds the inputs of a small world (terrain, monomers, velocity,
light, vent heat, agent shade), the base SimParams and settings, and the
state after stepping it: the monomer grid, velocity, pressure, temperature,
redox, divergence and the ledger.  The CPU tests check that the oracle still
reproduces them bit for bit (on any host ISA); the GPU tests check the CUDA
library against them.

Run from the repository root:  python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ribossome-v2_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ribo_oracle  # noqa: E402
import ribo_world as rw  # noqa: E402
import synth  # noqa: E402

OUT_FIELDS = {"chem": rw.CHEM, "velocity": rw.VELOCITY, "pressure": rw.PRESSURE, "temp": rw.TEMP,
              "redox": rw.REDOX, "divergence": rw.DIVERGENCE, "vel_smooth": rw.VEL_SMOOTH}
IN_FIELDS = {"gamma": rw.GAMMA, "chem_in": rw.CHEM, "velocity_in": rw.VELOCITY, "light": rw.LIGHT,
             "heat": rw.HEAT, "shade": rw.SHADE}

# name, grid, fluid, cfg kwargs, params, settings, batches
CASES = [
    ("g32_reference_defaults", 32, None, {}, dict(seed=11), {}, [5, 3]),
    ("g48_full_step_mg16", 48, None, dict(mg_min_size=16, mg_pre=3, mg_post=3),
     dict(seed=12, dt=1.0, transport_every=1, sun_heat=0.0), dict(fluid_substep=1, mg_cycles=2), [1, 2]),
    ("g64_f32_reactions_sun_vent", 64, 32, {},
     dict(seed=13, dt=0.2, aggregation=0.05, monomer_pressure=1.5, cohesion=0.5, thermal_activation=1.0,
          activation_decay=0.02, direct_photoactivation=0.5, settle=1.0, day_period=300.0, transport_every=1),
     dict(fluid_substep=1), [2, 2]),
    ("r64x32_jacobi_sparse", (64, 32), None, {}, dict(seed=14, dt=1.0, transport_every=2),
     dict(fluid_substep=1, multigrid=0, jacobi_iters=12), [3, 3]),
]


def make_inputs(grid, fluid, seed):
    inp = synth.make_world_inputs(grid, fluid, seed=seed, monomer_mean=5.0, rock_frac=0.15)
    gw, gh = (grid, grid) if isinstance(grid, int) else grid
    fw, fh = (gw, gh) if fluid is None else ((fluid, fluid) if isinstance(fluid, int) else fluid)
    rng = np.random.default_rng(seed)
    heat = np.zeros((fh, fw, 2), np.float32)
    heat[1:3, fw // 2 - 2:fw // 2 + 2, 0] = 3000.0
    heat[1:3, fw // 2 - 2:fw // 2 + 2, 1] = 80.0
    shade = rng.integers(0, 200, size=(2, gh // 2, gw // 2)).astype(np.uint32)
    inp[rw.HEAT] = heat
    inp[rw.SHADE] = shade
    # a few over-full cells exercise the squeeze rule
    chem = inp[rw.CHEM].reshape(gh, gw, 4).copy()
    chem[gh // 3, gw // 3] = [30 | (25 << 16), 20, 40 << 16, 15 | (15 << 16)]
    inp[rw.CHEM] = chem
    return inp


def run_case(world, case, inputs):
    name, grid, fluid, cfgkw, params, settings, batches = case
    world.seed_inputs(inputs)
    for k, v in params.items():
        setattr(world.params, k, v)
    for k, v in settings.items():
        setattr(world.settings, k, v)
    for b in batches:
        world.encode_steps(b)
    return {k: world.read(f) for k, f in OUT_FIELDS.items()}, world.ledger_blocking()


def main():
    for case in CASES:
        name, grid, fluid, cfgkw, params, settings, batches = case
        seed = params["seed"]
        inputs = make_inputs(grid, fluid, seed)
        o = ribo_oracle.OracleWorld(grid, fluid, seed=seed, **cfgkw)
        base = o.params.copy()
        outs, ledger = run_case(o, case, inputs)
        for k, v in params.items():
            setattr(base, k, v)
        data = {f"in_{k}": inputs[f] for k, f in IN_FIELDS.items() if f in inputs}
        data.update({f"out_{k}": v for k, v in outs.items()})
        data["ledger"] = np.array(list(ledger.act) + list(ledger.spent) + list(ledger.held), np.uint32)
        data["params"] = np.frombuffer(bytes(base), np.uint8)
        st = rw.WorldSettings(1, 2, 1, 1, 128)
        for k, v in settings.items():
            setattr(st, k, v)
        data["settings"] = np.frombuffer(bytes(st), np.uint8)
        data["cfg"] = np.frombuffer(bytes(o.cfg), np.uint8)
        data["batches"] = np.array(batches, np.int32)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
        print(name, {k: v.shape for k, v in outs.items()}, ledger.total())


if __name__ == "__main__":
    main()
