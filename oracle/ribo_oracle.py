"""ctypes wrapper of the CPU oracle -- test infrastructure only.

`OracleWorld` mirrors `ribo_world.World` (same fields, same step contract)
on top of oracle/_build/libribo_oracle.so, the CPU restatement of the
reference's world-step passes.  Only the test suite, the smoke check and
bench.py's CPU-baseline leg use it, as the checker; the product never does.
"""
from __future__ import annotations

import ctypes
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "ribossome-v2_gb300"))
sys.path.insert(0, HERE)
import ribo_world as rw  # noqa: E402  (ABI structs and field ids only)

from build_oracle import build as _build  # noqa: E402

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(_build())
        vp = ctypes.c_void_p
        P = ctypes.POINTER
        sig = {
            "orc_create": ([P(rw.WorldCfg)], vp),
            "orc_destroy": ([vp], None),
            "orc_set_settings": ([vp, P(rw.WorldSettings)], None),
            "orc_upload": ([vp, ctypes.c_int, vp, ctypes.c_size_t], ctypes.c_int),
            "orc_read": ([vp, ctypes.c_int, vp, ctypes.c_size_t], ctypes.c_int),
            "orc_step": ([vp, P(rw.SimParams), ctypes.c_uint32], None),
            "orc_ledger": ([vp, P(ctypes.c_uint32)], None),
            "orc_num_levels": ([vp], ctypes.c_int),
            "orc_set_threads": ([ctypes.c_int], None),
            "orc_get_threads": ([], ctypes.c_int),
            "orc_pass": ([vp, P(rw.SimParams), ctypes.c_int], None),
            "orc_paint": ([vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32], None),
            "orc_read_vel_b": ([vp, vp, ctypes.c_size_t], ctypes.c_int),
            "orc_write_vel_b": ([vp, vp, ctypes.c_size_t], ctypes.c_int),
            "orc_exp": ([ctypes.c_float], ctypes.c_float),
            "orc_log": ([ctypes.c_float], ctypes.c_float),
            "orc_pow": ([ctypes.c_float, ctypes.c_float], ctypes.c_float),
            "orc_sin": ([ctypes.c_float], ctypes.c_float),
            "orc_pcg4d": ([ctypes.c_uint32] * 4 + [P(ctypes.c_uint32)], None),
        }
        for name, (a, r) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = a
            fn.restype = r
        _lib = lib
    return _lib


def set_threads(n: int):
    load().orc_set_threads(n)


def get_threads() -> int:
    return load().orc_get_threads()


def _f32(x) -> float:
    return float(np.float32(x))


def derive_step_params(base: "rw.SimParams", settings: "rw.WorldSettings", steps: int):
    """World::encode_steps per-step copies (src/world/mod.rs:1422-1445),
    restated in Python with SimParams::daylight / sun_slope_at
    (src/params.rs:497-534)."""
    substep = min(max(settings.fluid_substep, 1), 4)
    b = base.copy()
    b.fluid_dt = _f32(np.float32(b.dt) * np.float32(substep))
    b.fluid_enabled = 1 if settings.fluid_enabled else 0

    def day_phase(epoch):
        x = epoch / float(np.float32(b.day_period))
        ph = x - math.trunc(x)
        frac = min(max(float(np.float32(b.day_fraction)), 0.05), 1.0)
        return ph < frac, ph / frac

    def daylight(epoch):
        if b.day_period < 1.0:
            return 1.0
        day, ph = day_phase(epoch)
        if not day:
            return 0.0
        return _f32(max(math.sin(math.pi * ph), 0.0))

    def slope(epoch):
        if b.day_period < 1.0:
            return 0.0
        day, ph = day_phase(epoch)
        a = min(max(float(np.float32(b.sun_angle)), 0.0), 85.0) * (math.pi / 180.0)
        if not day:
            ph = 1.0
        return _f32(math.tan((ph - 0.5) * 2.0 * a))

    out = (rw.SimParams * steps)()
    for i in range(steps):
        p = b.copy()
        p.epoch = (b.epoch + i) & 0xFFFFFFFF
        if i > 0:
            p.spawn_count = 0
        p.sun_now = daylight(p.epoch) if b.uv_strength > 0.0 else 0.0
        p.sun_slope = slope(p.epoch)
        out[i] = p
    return out


class OracleWorld:
    """CPU restatement with the interface of ribo_world.World."""

    def __init__(self, grid, fluid=None, seed: int = 1, *, world_units_per_cell: int = 30,
                 mg_min_size: int = 8, mg_pre: int = 2, mg_post: int = 2, mg_coarse: int = 30):
        lib = load()
        gw, gh = (grid, grid) if isinstance(grid, int) else grid
        if fluid is None:
            fluid = (gw, gh)
        fw, fh = (fluid, fluid) if isinstance(fluid, int) else fluid
        self.cfg = rw.WorldCfg(gw, gh, fw, fh, world_units_per_cell, mg_min_size, mg_pre, mg_post, mg_coarse, 0)
        self.gw, self.gh, self.fw, self.fh = gw, gh, fw, fh
        self._h = lib.orc_create(ctypes.byref(self.cfg))
        self._lib = lib
        self.params = _default_params(seed)
        self.settings = _default_settings()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    field_shape = rw.World.field_shape

    def num_levels(self) -> int:
        return self._lib.orc_num_levels(self._h)

    def upload(self, field: int, array):
        shape, dt = self.field_shape(field)
        a = np.ascontiguousarray(array, dtype=dt).reshape(shape)
        if self._lib.orc_upload(self._h, field, a.ctypes.data, a.nbytes):
            raise ValueError(f"oracle upload {field}")

    def read(self, field: int) -> np.ndarray:
        shape, dt = self.field_shape(field)
        a = np.empty(shape, dtype=dt)
        if self._lib.orc_read(self._h, field, a.ctypes.data, a.nbytes):
            raise ValueError(f"oracle read {field}")
        return a

    def read_cells_blocking(self):
        return self.read(rw.CHEM).reshape(-1)

    def seed_inputs(self, inputs: dict):
        rw.World.seed_inputs(self, inputs)

    def step(self, per_step):
        self._lib.orc_set_settings(self._h, ctypes.byref(self.settings))
        n = len(per_step)
        arr = per_step if isinstance(per_step, ctypes.Array) else (rw.SimParams * n)(*per_step)
        self._lib.orc_step(self._h, arr, n)

    def encode_steps(self, steps: int):
        steps = min(steps, rw.MAX_STEPS_PER_FRAME)
        if steps == 0:
            return
        per = derive_step_params(self.params, self.settings, steps)
        self.step(per)
        self.params.fluid_dt = per[0].fluid_dt
        self.params.fluid_enabled = per[0].fluid_enabled
        self.params.epoch = (self.params.epoch + steps) & 0xFFFFFFFF

    def run(self, steps: int):
        done = 0
        while done < steps:
            n = min(rw.MAX_STEPS_PER_FRAME, steps - done)
            self.encode_steps(n)
            done += n

    def run_pass(self, params: "rw.SimParams", which: int):
        self._lib.orc_set_settings(self._h, ctypes.byref(self.settings))
        self._lib.orc_pass(self._h, ctypes.byref(params), which)

    def encode_paint(self, cx: float, cy: float, radius: float, grains: int):
        self._lib.orc_paint(self._h, cx, cy, radius, grains)

    def ledger_blocking(self) -> "rw.Ledger":
        out = (ctypes.c_uint32 * 12)()
        self._lib.orc_ledger(self._h, out)
        return rw.Ledger.from_words(out)


# Reference defaults, restated independently of the CUDA library
# (src/params.rs:553-690 and src/world/mod.rs:117-134).
_DEFAULTS = dict(
    epoch=0, seed=1, dt=0.017, diffusion=12.0, settle=0.0, fluid_dt=float(np.float32(0.017) * np.float32(2.0)),
    fluid_decay=0.99, fluid_vorticity=7.7, fluid_viscosity=3.7, fumarole_count=0, uv_strength=3.0, uv_depth=0.0,
    fluid_enabled=1, fluid_obstacle_strength=1000.0, slope_steer_rate=210.0, cohesion=0.25, spawn_count=0,
    max_agents=0, death_probability=0.0006, spawn_energy=5.0, food_power=6.0, maintenance_cost=0.002,
    pairing_rate=3.0, mutation_rate=0.005, uv_damage=1.0, uptake_rate=0.0003, brownian=0.0, phoretic_gain=0.0,
    chain_stiffness=100.0, thermal_kt=0.1, motor_amplitude=0.4, rft_enabled=1, require_start=1, joint_coupling=0.0,
    hunger_regulation=1, pairing_cost=0.1, reactivation_rate=0.00001, swim_gain=2.0, bioturbation=0.39,
    bioturbation_cost=0.01, monomer_uv_absorb=0.3, sedimentation=0.0, direct_photoactivation=0.02,
    activation_decay=0.0, monomer_pressure=0.0, agent_fluid_push=0.001, swim_wobble=1.0, fluid_swim_only=0,
    motion_cost=0.06, bond_rate=0.05, bond_energy_share=0.1, bond_signal=0.5, aggregation=0.03, photo_yield=0.5,
    heat_kill=0.27, flow_coupling=0.9, inertia=0.0, death_energy_cap=1.0, chemo_yield=0.9, redox_decay=0.02,
    thermal_activation=0.045, denature_temp=2.0, day_period=8000.0, sun_slope=0.0, sun_now=1.0, sun_angle=80.0,
    day_fraction=0.75, metabolic_q10=2.0, metabolic_span=3.0, metabolic_ref=0.0, sun_heat=1.0,
    sediment_transport=1.9, sediment_threshold=0.5, sediment_settle=0.0, signal_mode=0.0, clock_mute=0.0,
    paint_x=0.0, paint_y=0.0, paint_radius=0.0, paint_grains=0.0, rest_angle_mult=1.0, protease_power=1.5,
    lysis_yield=0.7, protease_direct=0.5, joint_load=1.0, swim_grip=10.0, swim_memory=1.0, mouth_leak=0.3,
    leak_base=0.05, skin_uptake=0.1, death_metab=0.2, salvage=0.0, bond_matter_share=0.1, brownian_rot=0.0,
    transport_every=3, signal_crosstalk=0.1, flow_mass=0.0, chemo_take=0.008, vent_cycle_period=7000.0,
    vent_cycle_amp=0.91, sediment_cohesion=0.5, sediment_compaction=0.00001, rock_crumble=0.0001,
    lysis_matter=0.5, scramble_conduction=0, scramble_angles=0, scramble_response=0, scramble_amount=1.0,
    pairing_energy_half=0.5, pairing_min_energy=0.0, uv_mutation=0.0, heat_mutation=0.0, birth_crowding=80.0,
    photo_damage=0.005, naked_decay=0.005, store_loss=0.0001,
)


def _default_params(seed: int = 1) -> "rw.SimParams":
    p = rw.SimParams()
    for k, v in _DEFAULTS.items():
        setattr(p, k, v)
    p.seed = seed
    return p


def _default_settings() -> "rw.WorldSettings":
    """src/world/mod.rs:117-134: fluid on, substep 2, multigrid with one
    V-cycle, 128 Jacobi iterations, the light propagating one row per step
    with full sweeps every 10 steps when it does not; the light and the
    terrain stay frozen inputs unless a test turns their blocks on."""
    s = rw.WorldSettings(1, 2, 1, 1, 128)
    s.light_rows_per_step = 1
    s.light_interval = 10
    return s


default_params = _default_params
default_settings = _default_settings
