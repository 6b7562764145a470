"""Scene files on the GPU: a saved world loads back bit for bit and steps on
identically, and a file laid out like the reference's scenes (agent blocks,
parameters by name, unknown and missing names) loads into a world."""
import json
import struct

import numpy as np
import pytest

from helpers import assert_same

pytestmark = pytest.mark.gpu

FIELDS = ("CHEM", "GAMMA", "VELOCITY", "PRESSURE", "TEMP", "REDOX", "HEAT", "LIGHT", "SHADE")


def make_world(rw, synth, n, seed, fluid=None):
    w = rw.World(n, fluid, seed=seed, mg_min_size=16, mg_pre=3, mg_post=3)
    w.seed_inputs(synth.make_world_inputs(n, fluid, seed=seed, rubble_frac=0.1))
    w.params.dt = 1.0
    w.params.transport_every = 1
    w.settings.fluid_substep = 1
    w.settings.mg_cycles = 2
    return w


def test_save_load_round_trip_and_continuation(rw, tmp_path):
    import synth

    a = make_world(rw, synth, 128, 41)
    heat = np.zeros(a.field_shape(rw.HEAT)[0], np.float32)
    heat[10:14, 30:40, 0] = 300.0
    a.upload(rw.HEAT, heat)
    a.encode_steps(5)
    path = str(tmp_path / "world.ribo")
    a.save_scene(path)
    b = rw.World(128, seed=2, mg_min_size=16, mg_pre=3, mg_post=3)
    b.load_scene(path)
    for name in FIELDS:
        f = getattr(rw, name)
        assert_same(a.read(f), b.read(f), f"field {name} after load")
    assert bytes(a.params) == bytes(b.params)
    for k in ("fluid_enabled", "fluid_substep", "multigrid", "mg_cycles", "jacobi_iters"):
        assert getattr(a.settings, k) == getattr(b.settings, k), k
    a.encode_steps(4)
    b.encode_steps(4)
    for name in FIELDS:
        f = getattr(rw, name)
        assert_same(a.read(f), b.read(f), f"field {name} after 4 more steps")
    assert a.ledger_blocking() == b.ledger_blocking()


def block(rw, name, data):
    c = rw.lz4_compress(data)
    nb = name.encode()
    return struct.pack("<H", len(nb)) + nb + struct.pack("<Q", len(c) + 4) + struct.pack("<I", len(data)) + c


def test_loads_a_reference_layout_scene(rw, tmp_path):
    import synth

    n = 64
    src = make_world(rw, synth, n, 7)
    names = rw.sim_param_names()
    params = {k: float(getattr(src.params, k)) for k in names}
    params["epoch"] = 1234.0
    params["diffusion"] = 7.5
    params["a_parameter_that_no_longer_exists"] = 3.0
    del params["settle"]                                   # missing: takes the default
    header = {"versao": 2, "gravado": 0, "agentes": 1,
              "cfg": {"grid_size": n, "fluid_size": n, "world_units_per_cell": 30, "max_agents": 4096},
              "params": params,
              "settings": {"fluid_enabled": True, "fluid_substep": 1, "multigrid": True, "mg_cycles": 3,
                           "jacobi_iters": 64, "light_rows_per_step": 1, "light_interval": 10,
                           "terrain_enabled": True, "contact_enabled": True},
              "fumarolas": [], "interface": {"camera": [1, 2, 3]}, "tabela_orgaos": [{"nome": "olá"}]}
    h = json.dumps(header, indent=2).encode()
    out = b"RIBOSCN1" + struct.pack("<I", len(h)) + h
    out += block(rw, "slots", struct.pack("<I", 5))
    out += block(rw, "life_counters", bytes(32))
    out += block(rw, "agents", bytes(range(256)) * 3)      # agent blocks: not this path's, ignored
    rng = np.random.default_rng(9)
    vel = rng.standard_normal((n, n, 2)).astype(np.float32) * 0.1
    pres = rng.standard_normal((n, n)).astype(np.float32)
    temp = np.abs(rng.standard_normal((n, n))).astype(np.float32)
    chem = src.read(rw.CHEM)
    gamma = src.read(rw.GAMMA)
    out += block(rw, "chem", chem.tobytes()) + block(rw, "gamma", gamma.tobytes())
    out += block(rw, "velocity", vel.tobytes()) + block(rw, "pressure", pres.tobytes())
    out += block(rw, "temperature", temp.tobytes())
    path = tmp_path / "reference_layout.ribo"
    path.write_bytes(out)

    w = rw.World(n, seed=3, mg_min_size=16, mg_pre=3, mg_post=3)
    w.load_scene(str(path))
    assert_same(w.read(rw.CHEM), chem, "chem")
    assert_same(w.read(rw.GAMMA), gamma, "gamma")
    assert_same(w.read(rw.VELOCITY), vel, "velocity")
    assert_same(w.read(rw.PRESSURE), pres, "pressure")
    assert_same(w.read(rw.TEMP), temp, "temperature")
    assert w.params.epoch == 1234 and w.params.diffusion == np.float32(7.5)
    assert w.params.settle == rw.default_params().settle
    assert w.settings.mg_cycles == 3 and w.settings.jacobi_iters == 64 and w.settings.fluid_substep == 1
    w.encode_steps(2)                                       # and it steps
    assert rw.Ledger.from_cells(w.read_cells_blocking()) == w.ledger_blocking()


def test_rejects_another_world_size(rw, tmp_path):
    import synth

    a = make_world(rw, synth, 64, 1)
    path = str(tmp_path / "small.ribo")
    a.save_scene(path)
    b = rw.World(96, seed=1)
    with pytest.raises(rw.RiboError, match="another world size"):
        b.load_scene(path)
