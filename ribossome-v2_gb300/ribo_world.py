"""Python mirror of the reference's world-step API over the C ABI.

`World` follows the reference's `World` (src/world/mod.rs): it owns the
device state, exposes `params` (SimParams) and `settings` (WorldSettings),
`encode_steps(steps)` records steps and advances `params.epoch`, and
`ledger_blocking()` / `read_cells_blocking()` / `read_f32_blocking(field)`
read results back.  All compute runs in libribo_world.so (CUDA, sm_103a);
loading fails loudly when the library is missing -- there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os
import re
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
HEADER = os.path.join(REPO, "include", "ribo_world.h")
LIB_PATH = os.path.join(HERE, "_build", "libribo_world.so")

# ribo_field
CHEM, GAMMA, LIGHT, SLOPE, VELOCITY, PRESSURE, TEMP, REDOX, HEAT = range(9)
VEL_SMOOTH, SOLID_MASK, DIVERGENCE, FORCE_VECTORS, REDOX_EATEN, NET_FLUX, SHADE = range(9, 16)
PRESSURE_LO = 16

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "OVER_BUDGET", 4: "TIMEOUT", 5: "CUDA_ERROR"}
MAX_STEPS_PER_FRAME = 64


def _sim_param_fields():
    """The SimParams field list, read from the C header (one source of truth)."""
    text = open(HEADER).read()
    body = re.search(r"typedef struct ribo_sim_params \{(.*?)\} ribo_sim_params;", text, re.S).group(1)
    fields = []
    for ty, name in re.findall(r"^\s*(uint32_t|float)\s+(\w+);", body, re.M):
        fields.append((name, ctypes.c_uint32 if ty == "uint32_t" else ctypes.c_float))
    return fields


class SimParams(ctypes.Structure):
    _fields_ = _sim_param_fields()

    def copy(self) -> "SimParams":
        c = SimParams()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(SimParams))
        return c


assert ctypes.sizeof(SimParams) == 464, ctypes.sizeof(SimParams)


class WorldCfg(ctypes.Structure):
    _fields_ = [
        ("grid_w", ctypes.c_uint32), ("grid_h", ctypes.c_uint32),
        ("fluid_w", ctypes.c_uint32), ("fluid_h", ctypes.c_uint32),
        ("world_units_per_cell", ctypes.c_uint32), ("mg_min_size", ctypes.c_uint32),
        ("mg_pre", ctypes.c_uint32), ("mg_post", ctypes.c_uint32), ("mg_coarse", ctypes.c_uint32),
        ("precision_mode", ctypes.c_uint32), ("device", ctypes.c_uint32), ("no_graphs", ctypes.c_uint32),
        ("mg_cluster", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 3),
    ]


class WorldSettings(ctypes.Structure):
    _fields_ = [
        ("fluid_enabled", ctypes.c_uint32), ("fluid_substep", ctypes.c_uint32),
        ("multigrid", ctypes.c_uint32), ("mg_cycles", ctypes.c_uint32),
        ("jacobi_iters", ctypes.c_uint32), ("ledger_each_step", ctypes.c_uint32),
        ("mg_unfused", ctypes.c_uint32), ("transport_simple", ctypes.c_uint32),
        ("mixed_tol", ctypes.c_float), ("mixed_inner_tol", ctypes.c_float),
        ("mixed_max_outer", ctypes.c_uint32), ("mixed_max_inner", ctypes.c_uint32), ("mixed_alpha", ctypes.c_float),
        ("light_mode", ctypes.c_uint32), ("light_rows_per_step", ctypes.c_uint32), ("light_interval", ctypes.c_uint32),
        ("terrain_mode", ctypes.c_uint32),
    ]


class KernelTiming(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 40), ("launches", ctypes.c_uint32), ("ms", ctypes.c_float),
                ("bytes", ctypes.c_double)]


class ServerCfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_uint32), ("max_chunk_steps", ctypes.c_uint32), ("max_active", ctypes.c_uint32),
                ("reserved0", ctypes.c_uint32), ("hbm_budget_bytes", ctypes.c_uint64), ("reserved", ctypes.c_uint64 * 2)]


class Job(ctypes.Structure):
    _fields_ = [("world", WorldCfg), ("settings", WorldSettings), ("params", SimParams), ("steps", ctypes.c_uint32),
                ("reserved0", ctypes.c_uint32), ("user_tag", ctypes.c_uint64),
                ("inputs", ctypes.c_void_p * 17), ("outputs", ctypes.c_void_p * 17)]


class JobResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("user_tag", ctypes.c_uint64), ("status", ctypes.c_int32),
                ("steps", ctypes.c_uint32), ("ledger", ctypes.c_uint32 * 12), ("device_bytes", ctypes.c_uint64),
                ("t_submit_ms", ctypes.c_double), ("t_admit_ms", ctypes.c_double), ("t_done_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("pending", ctypes.c_uint64), ("active", ctypes.c_uint64), ("bytes_in_use", ctypes.c_uint64),
                ("world_steps", ctypes.c_uint64), ("iterations", ctypes.c_uint64), ("gpu_ms", ctypes.c_double)]


assert ctypes.sizeof(WorldSettings) == 68 and ctypes.sizeof(Job) == 888 and ctypes.sizeof(JobResult) == 104
assert ctypes.sizeof(ServerCfg) == 40


class RiboError(RuntimeError):
    pass


_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libribo_world.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RiboError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    sig = {
        "ribo_last_error": ([], ctypes.c_char_p),
        "ribo_sim_params_default": ([P(SimParams)], None),
        "ribo_world_settings_default": ([P(WorldSettings)], None),
        "ribo_world_create": ([P(WorldCfg), P(vp)], ctypes.c_int),
        "ribo_world_destroy": ([vp], None),
        "ribo_world_set_settings": ([vp, P(WorldSettings)], ctypes.c_int),
        "ribo_world_get_settings": ([vp, P(WorldSettings)], ctypes.c_int),
        "ribo_world_upload": ([vp, ctypes.c_int, vp, ctypes.c_size_t], ctypes.c_int),
        "ribo_world_paint_terrain": ([vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32], ctypes.c_int),
        "ribo_world_read": ([vp, ctypes.c_int, vp, ctypes.c_size_t], ctypes.c_int),
        "ribo_world_device_ptr": ([vp, ctypes.c_int, P(vp), P(ctypes.c_size_t)], ctypes.c_int),
        "ribo_world_step": ([vp, P(SimParams), ctypes.c_uint32], ctypes.c_int),
        "ribo_world_encode_steps": ([vp, P(SimParams), ctypes.c_uint32], ctypes.c_int),
        "ribo_derive_step_params": ([P(SimParams), P(WorldSettings), ctypes.c_uint32, P(SimParams)], ctypes.c_int),
        "ribo_world_ledger": ([vp, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_world_sync": ([vp], ctypes.c_int),
        "ribo_world_raise_status": ([vp, ctypes.c_uint32], ctypes.c_int),
        "ribo_selftest_bounded_wait": ([ctypes.c_uint32, ctypes.c_uint32, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_world_last_step_ms": ([vp, P(ctypes.c_float)], ctypes.c_int),
        "ribo_world_enable_kernel_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "ribo_world_read_kernel_timing": ([vp, P(KernelTiming), ctypes.c_uint32, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_kernel_launch_count": ([], ctypes.c_uint64),
        "ribo_world_save_scene": ([vp, ctypes.c_char_p, P(SimParams)], ctypes.c_int),
        "ribo_world_request_ledger": ([vp], ctypes.c_int),
        "ribo_world_poll_ledger": ([vp, P(ctypes.c_uint32), P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_world_load_scene": ([vp, ctypes.c_char_p, P(SimParams)], ctypes.c_int),
        "ribo_sim_param_name": ([ctypes.c_uint32], ctypes.c_char_p),
        "ribo_lz4_compress_bound": ([ctypes.c_size_t], ctypes.c_size_t),
        "ribo_lz4_compress": ([vp, ctypes.c_size_t, vp, ctypes.c_size_t, P(ctypes.c_size_t)], ctypes.c_int),
        "ribo_lz4_decompress": ([vp, ctypes.c_size_t, vp, ctypes.c_size_t, P(ctypes.c_size_t)], ctypes.c_int),
        "ribo_world_step_ledgers": ([vp, P(ctypes.c_uint32), ctypes.c_uint32], ctypes.c_int),
        "ribo_world_mark": ([vp, ctypes.c_uint32], ctypes.c_int),
        "ribo_world_elapsed_ms": ([vp, ctypes.c_uint32, ctypes.c_uint32, P(ctypes.c_float)], ctypes.c_int),
        "ribo_batch_create": ([ctypes.c_uint32, P(vp)], ctypes.c_int),
        "ribo_batch_destroy": ([vp], None),
        "ribo_batch_add": ([vp, vp], ctypes.c_int),
        "ribo_batch_remove": ([vp, vp], ctypes.c_int),
        "ribo_batch_size": ([vp], ctypes.c_uint32),
        "ribo_batch_step": ([vp, P(SimParams), ctypes.c_uint32], ctypes.c_int),
        "ribo_batch_encode_steps": ([vp, P(SimParams), ctypes.c_uint32], ctypes.c_int),
        "ribo_batch_step_ledgers": ([vp, P(ctypes.c_uint32), ctypes.c_uint32], ctypes.c_int),
        "ribo_batch_sync": ([vp], ctypes.c_int),
        "ribo_batch_mark": ([vp, ctypes.c_uint32], ctypes.c_int),
        "ribo_batch_elapsed_ms": ([vp, ctypes.c_uint32, ctypes.c_uint32, P(ctypes.c_float)], ctypes.c_int),
        "ribo_batch_autotune": ([vp, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_batch_set_tile_modes": ([vp, P(ctypes.c_uint32), ctypes.c_uint32], ctypes.c_int),
        "ribo_batch_step_ragged": ([vp, P(SimParams), ctypes.c_uint32, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_world_footprint": ([P(WorldCfg), P(ctypes.c_uint64)], ctypes.c_int),
        "ribo_world_solve_info": ([vp, P(ctypes.c_uint32), P(ctypes.c_uint32), P(ctypes.c_double)], ctypes.c_int),        "ribo_world_memory": ([vp, P(ctypes.c_uint64)], ctypes.c_int),
        "ribo_server_create": ([P(ServerCfg), P(vp)], ctypes.c_int),
        "ribo_server_destroy": ([vp], None),
        "ribo_server_submit": ([vp, P(Job), P(ctypes.c_uint64)], ctypes.c_int),
        "ribo_server_iterate": ([vp, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_server_drain": ([vp], ctypes.c_int),
        "ribo_server_results": ([vp, P(JobResult), ctypes.c_uint32, P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_server_get_stats": ([vp, P(ServerStats)], ctypes.c_int),
        "ribo_server_iterations": ([vp, P(ctypes.c_float), P(ctypes.c_uint32), P(ctypes.c_uint32), ctypes.c_uint32,
                                    P(ctypes.c_uint32)], ctypes.c_int),
        "ribo_batch_enable_kernel_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "ribo_batch_read_kernel_timing": ([vp, P(KernelTiming), ctypes.c_uint32, P(ctypes.c_uint32)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status: int, what: str = ""):
    if status != 0:
        msg = load_library().ribo_last_error().decode(errors="replace")
        raise RiboError(f"{what}: {STATUS.get(status, status)}: {msg}")


def kernel_launch_count() -> int:
    return int(load_library().ribo_kernel_launch_count())


def sim_param_names():
    """SimParams field names in order (the reference's to_named names)."""
    lib = load_library()
    out, i = [], 0
    while True:
        n = lib.ribo_sim_param_name(i)
        if n is None:
            return out
        out.append(n.decode())
        i += 1


def lz4_compress(data: bytes) -> bytes:
    """One LZ4 block (the scene files' block coder)."""
    lib = load_library()
    src = bytes(data)
    cap = lib.ribo_lz4_compress_bound(len(src))
    dst = ctypes.create_string_buffer(max(cap, 1))
    n = ctypes.c_size_t()
    check(lib.ribo_lz4_compress(src, len(src), dst, cap, ctypes.byref(n)), "lz4_compress")
    return dst.raw[:n.value]


def lz4_decompress(block: bytes, size: int) -> bytes:
    """Decodes one LZ4 block of `size` bytes."""
    lib = load_library()
    src = bytes(block)
    dst = ctypes.create_string_buffer(max(size, 1))
    n = ctypes.c_size_t()
    check(lib.ribo_lz4_decompress(src, len(src), dst, size, ctypes.byref(n)), "lz4_decompress")
    return dst.raw[:n.value]


def default_params(seed: int = 1) -> SimParams:
    p = SimParams()
    load_library().ribo_sim_params_default(ctypes.byref(p))
    p.seed = seed
    return p


def default_settings() -> WorldSettings:
    s = WorldSettings()
    load_library().ribo_world_settings_default(ctypes.byref(s))
    return s


def derive_step_params(base: SimParams, settings: WorldSettings, steps: int):
    out = (SimParams * steps)()
    check(load_library().ribo_derive_step_params(ctypes.byref(base), ctypes.byref(settings), steps, out), "derive")
    return out


@dataclass
class Ledger:
    """Exact matter count per channel (A U G C) and state (src/world/mod.rs:39-82)."""

    act: tuple
    spent: tuple
    held: tuple = (0, 0, 0, 0)

    def total(self) -> int:
        return sum(self.act) + sum(self.spent) + sum(self.held)

    def channel(self, ch: int) -> int:
        return self.act[ch] + self.spent[ch] + self.held[ch]

    @staticmethod
    def from_cells(cells: np.ndarray) -> "Ledger":
        c = np.asarray(cells, dtype=np.uint32).reshape(-1, 4)
        act = tuple(int(v) for v in (c & 0xFFFF).astype(np.uint64).sum(axis=0))
        spent = tuple(int(v) for v in (c >> 16).astype(np.uint64).sum(axis=0))
        return Ledger(act, spent)

    @staticmethod
    def from_words(w) -> "Ledger":
        w = [int(v) for v in w]
        return Ledger(tuple(w[0:4]), tuple(w[4:8]), tuple(w[8:12]))


class World:
    """One world on the GPU (the reference's `World`, hot-path part)."""

    def __init__(self, grid, fluid=None, seed: int = 1, *, world_units_per_cell: int = 30,
                 mg_min_size: int = 8, mg_pre: int = 2, mg_post: int = 2, mg_coarse: int = 30,
                 precision_mode: int = 0, device: int = 0, no_graphs: int = 0, mg_cluster: int = 0):
        lib = load_library()
        gw, gh = (grid, grid) if isinstance(grid, int) else grid
        if fluid is None:
            fluid = (gw, gh)
        fw, fh = (fluid, fluid) if isinstance(fluid, int) else fluid
        cfg = WorldCfg(gw, gh, fw, fh, world_units_per_cell, mg_min_size, mg_pre, mg_post, mg_coarse, precision_mode,
                       device, no_graphs, mg_cluster)
        self.cfg = cfg
        self.gw, self.gh, self.fw, self.fh = gw, gh, fw, fh
        h = ctypes.c_void_p()
        check(lib.ribo_world_create(ctypes.byref(cfg), ctypes.byref(h)), "ribo_world_create")
        self._h = h
        self._lib = lib
        self.params = default_params(seed)
        self.settings = default_settings()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ribo_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- sizes ----
    @property
    def cells(self) -> int:
        return self.gw * self.gh

    @property
    def fluid_cells(self) -> int:
        return self.fw * self.fh

    def field_shape(self, field: int):
        C, F, L = (self.gh, self.gw), (self.fh, self.fw), (self.gh // 2, self.gw // 2)
        return {
            CHEM: (C + (4,), np.uint32), GAMMA: (C, np.uint32), LIGHT: ((2,) + L, np.float32),
            SLOPE: (C + (2,), np.float32), VELOCITY: (F + (2,), np.float32), PRESSURE: (F, np.float32),
            TEMP: (F, np.float32), REDOX: (F, np.float32), HEAT: (F + (2,), np.float32),
            VEL_SMOOTH: (F + (2,), np.float32), SOLID_MASK: (F, np.uint32), DIVERGENCE: (F, np.float32),
            FORCE_VECTORS: (F + (2,), np.uint32), REDOX_EATEN: (F, np.uint32),
            NET_FLUX: ((self.fh + self.fw,), np.float32), SHADE: ((2,) + L, np.uint32), PRESSURE_LO: (F, np.float32),
        }[field]

    # ---- data movement ----
    def _sync_settings(self):
        check(self._lib.ribo_world_set_settings(self._h, ctypes.byref(self.settings)), "settings")

    def upload(self, field: int, array: np.ndarray):
        shape, dt = self.field_shape(field)
        a = np.ascontiguousarray(array, dtype=dt).reshape(shape)
        check(self._lib.ribo_world_upload(self._h, field, a.ctypes.data, a.nbytes), f"upload {field}")

    def encode_paint(self, cx: float, cy: float, radius: float, grains: int):
        """World::encode_paint (src/world/mod.rs:1220-1241): `grains` (at most 6)
        grains in every cell of the disc (centre and radius in cells); the
        monomers that no longer fit are evicted to a neighbour with room."""
        check(self._lib.ribo_world_paint_terrain(self._h, cx, cy, radius, grains), "paint")

    def read(self, field: int) -> np.ndarray:
        shape, dt = self.field_shape(field)
        a = np.empty(shape, dtype=dt)
        check(self._lib.ribo_world_read(self._h, field, a.ctypes.data, a.nbytes), f"read {field}")
        return a

    def device_ptr(self, field: int):
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        check(self._lib.ribo_world_device_ptr(self._h, field, ctypes.byref(p), ctypes.byref(n)), "device_ptr")
        return p.value, n.value

    def read_cells_blocking(self) -> np.ndarray:
        return self.read(CHEM).reshape(-1)

    def read_f32_blocking(self, field: int) -> np.ndarray:
        return self.read(field).reshape(-1).view(np.float32)

    # ---- stepping ----
    def step(self, per_step):
        """Records len(per_step) steps with explicit per-step SimParams."""
        self._sync_settings()
        n = len(per_step)
        arr = per_step if isinstance(per_step, ctypes.Array) else (SimParams * n)(*per_step)
        check(self._lib.ribo_world_step(self._h, arr, n), "ribo_world_step")

    def encode_steps(self, steps: int):
        """World::encode_steps: derives per-step params and advances params.epoch."""
        self._sync_settings()
        check(self._lib.ribo_world_encode_steps(self._h, ctypes.byref(self.params), steps), "encode_steps")

    def run(self, steps: int):
        """Steps in batches of MAX_STEPS_PER_FRAME, like tests/conservation.rs::run."""
        done = 0
        while done < steps:
            n = min(MAX_STEPS_PER_FRAME, steps - done)
            self.encode_steps(n)
            done += n

    def sync(self):
        check(self._lib.ribo_world_sync(self._h), "sync")

    def last_step_ms(self) -> float:
        ms = ctypes.c_float()
        check(self._lib.ribo_world_last_step_ms(self._h, ctypes.byref(ms)), "last_step_ms")
        return ms.value

    def enable_kernel_timing(self, on: bool = True):
        check(self._lib.ribo_world_enable_kernel_timing(self._h, 1 if on else 0), "kernel timing")

    def read_kernel_timing(self):
        """[(name, launches, ms, algorithmic bytes)] of the last step call."""
        cap = 128
        arr = (KernelTiming * cap)()
        n = ctypes.c_uint32()
        check(self._lib.ribo_world_read_kernel_timing(self._h, arr, cap, ctypes.byref(n)), "read timing")
        return [(arr[i].name.decode(), arr[i].launches, arr[i].ms, arr[i].bytes) for i in range(min(n.value, cap))]

    def step_ledgers(self, n: int):
        """Ledgers after each of the last call's n steps (settings.ledger_each_step)."""
        out = (ctypes.c_uint32 * (12 * n))()
        check(self._lib.ribo_world_step_ledgers(self._h, out, n), "step ledgers")
        return [Ledger.from_words(out[12 * i:12 * i + 12]) for i in range(n)]

    def mark(self, slot: int):
        check(self._lib.ribo_world_mark(self._h, slot), "mark")

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = ctypes.c_float()
        check(self._lib.ribo_world_elapsed_ms(self._h, a, b, ctypes.byref(ms)), "elapsed")
        return ms.value

    def solve_info(self):
        """(outer steps, CG iterations, relative residual) of the last mixed-precision solve."""
        o, i, r = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        check(self._lib.ribo_world_solve_info(self._h, ctypes.byref(o), ctypes.byref(i), ctypes.byref(r)), "solve_info")
        return o.value, i.value, r.value

    def request_ledger(self):
        """encode_ledger_readback: an asynchronous ledger of the state after the work recorded so far."""
        check(self._lib.ribo_world_request_ledger(self._h), "request_ledger")

    def poll_ledger(self):
        """poll_ledger: the requested ledger once it has arrived, else None (never waits)."""
        out = (ctypes.c_uint32 * 12)()
        ready = ctypes.c_uint32()
        check(self._lib.ribo_world_poll_ledger(self._h, out, ctypes.byref(ready)), "poll_ledger")
        return Ledger.from_words(out) if ready.value else None

    def ledger_blocking(self) -> Ledger:
        out = (ctypes.c_uint32 * 12)()
        check(self._lib.ribo_world_ledger(self._h, out), "ledger")
        return Ledger.from_words(out)

    # ---- scenes (src/world/snapshot.rs) ----
    def save_scene(self, path: str):
        """Writes the world (blocks, params, settings) as a .ribo scene file."""
        self._sync_settings()
        check(self._lib.ribo_world_save_scene(self._h, os.fsencode(path), ctypes.byref(self.params)), "save_scene")

    def load_scene(self, path: str):
        """Loads a .ribo scene of this world's size: blocks, params and settings."""
        p = SimParams()
        check(self._lib.ribo_world_load_scene(self._h, os.fsencode(path), ctypes.byref(p)), "load_scene")
        self.params = p
        check(self._lib.ribo_world_get_settings(self._h, ctypes.byref(self.settings)), "get_settings")

    def seed_inputs(self, inputs: dict):
        """Uploads a dict {field: array} (e.g. from synth.make_world_inputs)."""
        for f in (GAMMA, CHEM, LIGHT, VELOCITY, PRESSURE, TEMP, REDOX, HEAT, SHADE, FORCE_VECTORS, REDOX_EATEN):
            if f in inputs:
                self.upload(f, inputs[f])


class Batch:
    """Worlds advanced in lock step: every pass is one launch over all members.

    Members keep their own state and settings (World.settings is pushed to
    the library at every step call); each member's results are the bits it
    would get stepped alone with the same parameters.
    """

    def __init__(self, worlds=(), device: int = 0):
        lib = load_library()
        h = ctypes.c_void_p()
        check(lib.ribo_batch_create(device, ctypes.byref(h)), "ribo_batch_create")
        self._h = h
        self._lib = lib
        self.worlds = []
        for w in worlds:
            self.add(w)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ribo_batch_destroy(self._h)
            self._h = None
            self.worlds = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.worlds)

    def add(self, w: World):
        check(self._lib.ribo_batch_add(self._h, w._h), "ribo_batch_add")
        self.worlds.append(w)

    def remove(self, w: World):
        check(self._lib.ribo_batch_remove(self._h, w._h), "ribo_batch_remove")
        self.worlds.remove(w)

    def _sync_settings(self):
        for w in self.worlds:
            w._sync_settings()

    def step(self, per_world_steps):
        """per_world_steps[k] = the k-th member's list of per-step SimParams (same length for all)."""
        self._sync_settings()
        n = len(per_world_steps[0]) if per_world_steps else 0
        flat = [p for steps in per_world_steps for p in steps]
        assert len(flat) == n * len(self.worlds)
        arr = (SimParams * len(flat))(*flat)
        check(self._lib.ribo_batch_step(self._h, arr, n), "ribo_batch_step")

    def encode_steps(self, steps: int):
        """ribo_world_encode_steps for every member, advancing each member's params.epoch."""
        self._sync_settings()
        arr = (SimParams * len(self.worlds))(*[w.params for w in self.worlds])
        check(self._lib.ribo_batch_encode_steps(self._h, arr, steps), "ribo_batch_encode_steps")
        for w, p in zip(self.worlds, arr):
            w.params = p.copy()

    def run(self, steps: int):
        done = 0
        while done < steps:
            n = min(MAX_STEPS_PER_FRAME, steps - done)
            self.encode_steps(n)
            done += n

    def step_ledgers(self, n: int):
        """[member][step] Ledger after each of the last call's n steps."""
        N = len(self.worlds)
        out = (ctypes.c_uint32 * (12 * n * N))()
        check(self._lib.ribo_batch_step_ledgers(self._h, out, n), "batch step ledgers")
        return [[Ledger.from_words(out[12 * (k * n + i):12 * (k * n + i) + 12]) for i in range(n)] for k in range(N)]

    def sync(self):
        check(self._lib.ribo_batch_sync(self._h), "batch sync")

    def mark(self, slot: int):
        check(self._lib.ribo_batch_mark(self._h, slot), "mark")

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = ctypes.c_float()
        check(self._lib.ribo_batch_elapsed_ms(self._h, a, b, ctypes.byref(ms)), "elapsed")
        return ms.value

    def autotune(self):
        modes = (ctypes.c_uint32 * 8)()
        check(self._lib.ribo_batch_autotune(self._h, modes), "autotune")
        return list(modes)

    def set_tile_modes(self, modes):
        arr = (ctypes.c_uint32 * len(modes))(*modes)
        check(self._lib.ribo_batch_set_tile_modes(self._h, arr, len(modes)), "tile modes")

    def enable_kernel_timing(self, on: bool = True):
        check(self._lib.ribo_batch_enable_kernel_timing(self._h, 1 if on else 0), "kernel timing")

    def read_kernel_timing(self):
        cap = 128
        arr = (KernelTiming * cap)()
        n = ctypes.c_uint32()
        check(self._lib.ribo_batch_read_kernel_timing(self._h, arr, cap, ctypes.byref(n)), "read timing")
        return [(arr[i].name.decode(), arr[i].launches, arr[i].ms, arr[i].bytes) for i in range(min(n.value, cap))]


def world_footprint(grid, fluid=None, mg_min_size: int = 8) -> int:
    """Device bytes a world of this configuration allocates (no GPU needed)."""
    gw, gh = (grid, grid) if isinstance(grid, int) else grid
    fw, fh = (gw, gh) if fluid is None else ((fluid, fluid) if isinstance(fluid, int) else fluid)
    cfg = WorldCfg(gw, gh, fw, fh, 30, mg_min_size)
    out = ctypes.c_uint64()
    check(load_library().ribo_world_footprint(ctypes.byref(cfg), ctypes.byref(out)), "footprint")
    return out.value


class Server:
    """World-step jobs served with continuous batching under an HBM budget."""

    def __init__(self, hbm_budget_bytes: int, max_chunk_steps: int = 16, max_active: int = 0, device: int = 0):
        lib = load_library()
        cfg = ServerCfg(device, max_chunk_steps, max_active, 0, hbm_budget_bytes)
        h = ctypes.c_void_p()
        check(lib.ribo_server_create(ctypes.byref(cfg), ctypes.byref(h)), "ribo_server_create")
        self._h = h
        self._lib = lib
        self.device = device
        self._keep = {}  # job id -> (job struct, input arrays, output arrays)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ribo_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, grid, fluid=None, *, steps: int, params: SimParams, settings: WorldSettings = None,
               inputs: dict = None, outputs=(), mg_min_size: int = 8, mg_pre: int = 2, mg_post: int = 2,
               mg_coarse: int = 30, user_tag: int = 0, precision_mode: int = 0) -> int:
        """Queues a job; `outputs` lists the fields returned with its result.
        precision_mode 1 solves every step's pressure to the mixed-precision
        tolerance."""
        gw, gh = (grid, grid) if isinstance(grid, int) else grid
        fw, fh = (gw, gh) if fluid is None else ((fluid, fluid) if isinstance(fluid, int) else fluid)
        j = Job()
        j.world = WorldCfg(gw, gh, fw, fh, 30, mg_min_size, mg_pre, mg_post, mg_coarse, precision_mode, self.device, 0)
        j.settings = settings if settings is not None else default_settings()
        j.params = params
        j.steps = steps
        j.user_tag = user_tag
        shapes = _field_shapes(gw, gh, fw, fh)
        keep_in = []
        for f, arr in (inputs or {}).items():
            shape, dt = shapes[f]
            a = np.ascontiguousarray(arr, dtype=dt).reshape(shape)
            keep_in.append(a)
            j.inputs[f] = a.ctypes.data
        outs = {}
        for f in outputs:
            shape, dt = shapes[f]
            outs[f] = np.zeros(shape, dtype=dt)
            j.outputs[f] = outs[f].ctypes.data
        jid = ctypes.c_uint64()
        check(self._lib.ribo_server_submit(self._h, ctypes.byref(j), ctypes.byref(jid)), "ribo_server_submit")
        self._keep[jid.value] = (j, outs)
        return jid.value

    def iterate(self) -> int:
        a = ctypes.c_uint32()
        check(self._lib.ribo_server_iterate(self._h, ctypes.byref(a)), "ribo_server_iterate")
        return a.value

    def drain(self):
        check(self._lib.ribo_server_drain(self._h), "ribo_server_drain")

    def results(self):
        """[(JobResult, {field: array})] of the jobs finished since the last call."""
        cap = 256
        out = []
        while True:
            arr = (JobResult * cap)()
            n = ctypes.c_uint32()
            check(self._lib.ribo_server_results(self._h, arr, cap, ctypes.byref(n)), "results")
            for i in range(n.value):
                r = JobResult()
                ctypes.memmove(ctypes.byref(r), ctypes.byref(arr[i]), ctypes.sizeof(JobResult))
                _, outs = self._keep.pop(r.id, (None, {}))
                out.append((r, outs))
            if n.value < cap:
                return out

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(self._lib.ribo_server_get_stats(self._h, ctypes.byref(s)), "stats")
        return s

    def iterations(self):
        """[(device ms, steps, resident jobs)] per iteration since the last call."""
        cap = 4096
        out = []
        while True:
            ms = (ctypes.c_float * cap)()
            st = (ctypes.c_uint32 * cap)()
            ac = (ctypes.c_uint32 * cap)()
            n = ctypes.c_uint32()
            check(self._lib.ribo_server_iterations(self._h, ms, st, ac, cap, ctypes.byref(n)), "iterations")
            out += [(ms[i], st[i], ac[i]) for i in range(n.value)]
            if n.value < cap:
                return out


def _field_shapes(gw, gh, fw, fh):
    C, F, L = (gh, gw), (fh, fw), (gh // 2, gw // 2)
    return {
        CHEM: (C + (4,), np.uint32), GAMMA: (C, np.uint32), LIGHT: ((2,) + L, np.float32),
        SLOPE: (C + (2,), np.float32), VELOCITY: (F + (2,), np.float32), PRESSURE: (F, np.float32),
        TEMP: (F, np.float32), REDOX: (F, np.float32), HEAT: (F + (2,), np.float32),
        VEL_SMOOTH: (F + (2,), np.float32), SOLID_MASK: (F, np.uint32), DIVERGENCE: (F, np.float32),
        FORCE_VECTORS: (F + (2,), np.uint32), REDOX_EATEN: (F, np.uint32),
        NET_FLUX: ((fh + fw,), np.float32), SHADE: ((2,) + L, np.uint32), PRESSURE_LO: (F, np.float32),
    }
