"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py):
the oracle must reproduce them on any host (CPU test), and the CUDA library
must reproduce them bit for bit (GPU test)."""
import ctypes
import glob
import os

import numpy as np
import pytest

import ribo_world as rw
from helpers import assert_same

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
IN_FIELDS = {"gamma": rw.GAMMA, "chem_in": rw.CHEM, "velocity_in": rw.VELOCITY, "light": rw.LIGHT,
             "heat": rw.HEAT, "shade": rw.SHADE}
OUT_FIELDS = {"chem": rw.CHEM, "velocity": rw.VELOCITY, "pressure": rw.PRESSURE, "temp": rw.TEMP,
              "redox": rw.REDOX, "divergence": rw.DIVERGENCE, "vel_smooth": rw.VEL_SMOOTH}


def replay(make_world, path):
    z = np.load(path)
    cfg = rw.WorldCfg.from_buffer_copy(z["cfg"].tobytes())
    w = make_world(cfg)
    for k, f in IN_FIELDS.items():
        if f"in_{k}" in z:
            w.upload(f, z[f"in_{k}"])
    w.params = rw.SimParams.from_buffer_copy(z["params"].tobytes())
    # fixtures made before the mixed-precision fields existed hold a shorter
    # record; those fields are zero (= their defaults)
    sb = z["settings"].tobytes()
    w.settings = rw.WorldSettings.from_buffer_copy(sb + bytes(ctypes.sizeof(rw.WorldSettings) - len(sb)))
    for b in z["batches"]:
        w.encode_steps(int(b))
    for k, f in OUT_FIELDS.items():
        assert_same(w.read(f), z[f"out_{k}"], f"{os.path.basename(path)}: {k}")
    led = w.ledger_blocking()
    assert list(led.act) + list(led.spent) + list(led.held) == [int(v) for v in z["ledger"]]


def test_fixtures_exist():
    assert len(FIXTURES) >= 4


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_reproduces_golden(ro, path):
    def make(cfg):
        return ro.OracleWorld((cfg.grid_w, cfg.grid_h), (cfg.fluid_w, cfg.fluid_h), seed=1,
                              world_units_per_cell=cfg.world_units_per_cell, mg_min_size=cfg.mg_min_size,
                              mg_pre=cfg.mg_pre, mg_post=cfg.mg_post, mg_coarse=cfg.mg_coarse)

    replay(make, path)


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_cuda_reproduces_golden(rw, path):
    def make(cfg):
        return rw.World((cfg.grid_w, cfg.grid_h), (cfg.fluid_w, cfg.fluid_h), seed=1,
                        world_units_per_cell=cfg.world_units_per_cell, mg_min_size=cfg.mg_min_size,
                        mg_pre=cfg.mg_pre, mg_post=cfg.mg_post, mg_coarse=cfg.mg_coarse)

    replay(make, path)
