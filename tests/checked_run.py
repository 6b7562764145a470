"""Child process of test_checked_gpu.py: steps small worlds on the
bounds-checked library (_build/checked/libribo_world.so) and on the oracle,
compares every state field bit for bit, and fails if any kernel index check
fired (ribo_world_sync reports it).  Prints "ok" at the end."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (os.path.join(ROOT, "ribossome-v2_gb300"), os.path.join(ROOT, "oracle"), HERE):
    sys.path.insert(0, p)

import build  # noqa: E402
import ribo_oracle  # noqa: E402
import ribo_world as rw  # noqa: E402
import synth  # noqa: E402
from helpers import compare_worlds  # noqa: E402

rw.load_library(build.CHECKED_LIB)
ribo_oracle.load()

# grid, fluid, synth kwargs, params
CASES = [
    (64, None, {}, {}),
    ((96, 48), None, dict(rock_frac=0.2, monomer_mean=9.0), dict(aggregation=0.05, cohesion=0.6)),
    (64, 32, dict(rubble_frac=0.2), dict(monomer_pressure=2.0)),
    (48, None, dict(max_disp=2.5), {}),
]
for k, (grid, fluid, skw, params) in enumerate(CASES):
    inputs = synth.make_world_inputs(grid, fluid, seed=900 + k, **skw)
    g = rw.World(grid, fluid, seed=900 + k, mg_min_size=8, mg_pre=3, mg_post=3)
    o = ribo_oracle.OracleWorld(grid, fluid, seed=900 + k, mg_min_size=8, mg_pre=3, mg_post=3)
    for w in (g, o):
        w.seed_inputs(inputs)
        w.params.dt = 1.0
        w.params.transport_every = 1
        w.params.sun_heat = 0.0
        for name, v in params.items():
            setattr(w.params, name, v)
        w.settings.fluid_substep = 1
        w.settings.mg_cycles = 2
        w.encode_steps(3)
    g.sync()  # raises if an index check fired
    compare_worlds(g, o, f"checked build, case {k}")
    g.close()
print("ok")
