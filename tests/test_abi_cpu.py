"""The C-ABI library without a GPU: it loads, exports every symbol the
header declares, its host-side logic matches the reference, and device
calls fail with an error code instead of crashing."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names += re.findall(r"^[a-z_0-9 ]+\*?\s*\**(ribo_\w+)\(", text, re.M)
    return sorted(set(names))


def c_struct_fields(name):
    text = open(os.path.join(ROOT, "include", "ribo_world.h")).read()
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", text, re.S).group(1)
    fields = []
    for line in body.splitlines():
        line = line.split("//")[0].strip()
        if not line:
            continue
        decl = line.rstrip(";").split(None, 1)[1]
        fields += [re.sub(r"\[.*\]", "", f).strip() for f in decl.split(",")]
    return fields


def test_rust_binding_matches_header():
    """The Rust binding (rust/src/lib.rs) declares only functions the header
    declares, and its mirrored structs have the header's fields in order."""
    rs = open(os.path.join(ROOT, "rust", "src", "lib.rs")).read()
    fns = re.findall(r"pub fn (ribo_\w+)\(", rs)
    assert fns and not [f for f in fns if f not in declared_functions()]
    for c_name, rs_name in (("ribo_world_cfg", "RiboWorldCfg"), ("ribo_world_settings", "RiboWorldSettings")):
        body = re.search(r"pub struct " + rs_name + r" \{(.*?)\}", rs, re.S).group(1)
        rs_fields = re.findall(r"pub (\w+):", body)
        assert rs_fields == c_struct_fields(c_name), (c_name, rs_fields, c_struct_fields(c_name))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("ribo_world_create", "ribo_world_step", "ribo_world_encode_steps", "ribo_world_ledger",
              "ribo_world_upload", "ribo_world_read", "ribo_world_destroy", "ribo_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(rw):
    lib = rw.load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", rw.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(lib, n)


def test_sim_params_layout_and_defaults(rw, ro):
    assert ctypes.sizeof(rw.SimParams) == 464
    assert len(rw.SimParams._fields_) == 116
    a = rw.default_params(7)
    b = ro.default_params(7)
    for name, _ in rw.SimParams._fields_:
        assert getattr(a, name) == getattr(b, name), name
    s = rw.default_settings()
    assert (s.fluid_enabled, s.fluid_substep, s.multigrid, s.mg_cycles, s.jacobi_iters) == (1, 2, 1, 1, 128)


@pytest.mark.parametrize("day_period,uv", [(8000.0, 3.0), (0.0, 3.0), (400.0, 0.0), (37.5, 1.0)])
def test_derive_step_params_matches_encode_steps(rw, ro, day_period, uv):
    base = rw.default_params(3)
    base.epoch = 4000000000 - 20
    base.day_period = day_period
    base.uv_strength = uv
    base.dt = 0.25
    st = rw.default_settings()
    st.fluid_substep = 3
    a = rw.derive_step_params(base, st, 64)
    b = ro.derive_step_params(base, st, 64)
    for i in range(64):
        for name, _ in rw.SimParams._fields_:
            va, vb = getattr(a[i], name), getattr(b[i], name)
            assert va == vb or (np.isnan(va) and np.isnan(vb)), (i, name, va, vb)
        assert a[i].epoch == (base.epoch + i) & 0xFFFFFFFF
        assert a[i].fluid_dt == np.float32(0.25) * np.float32(3)


def test_invalid_arguments_are_rejected(rw):
    lib = rw.load_library()
    h = ctypes.c_void_p()
    cfg = rw.WorldCfg(100, 100, 30, 30)  # not an integer ratio
    assert lib.ribo_world_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert b"ratio" in lib.ribo_last_error()
    cfg = rw.WorldCfg(1, 1, 1, 1)
    assert lib.ribo_world_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert lib.ribo_world_step(None, None, 1) == 1
    cfg = rw.WorldCfg(64, 64, 64, 64)
    cfg.mg_cluster = 4  # 0, 1, 8 or 16
    n = ctypes.c_uint64()
    assert lib.ribo_world_footprint(ctypes.byref(cfg), ctypes.byref(n)) == 1
    assert b"mg_cluster" in lib.ribo_last_error()


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_create_without_gpu_reports_cuda_error(rw):
    with pytest.raises(rw.RiboError) as e:
        rw.World(32)
    assert "CUDA_ERROR" in str(e.value)


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_batch_without_gpu_reports_cuda_error(rw):
    with pytest.raises(rw.RiboError) as e:
        rw.Batch()
    assert "CUDA_ERROR" in str(e.value)


def test_batch_null_arguments_are_rejected(rw):
    lib = rw.load_library()
    assert lib.ribo_batch_create(0, None) == 1
    assert lib.ribo_batch_add(None, None) == 1
    assert lib.ribo_batch_remove(None, None) == 1
    assert lib.ribo_batch_step(None, None, 1) == 1
    assert lib.ribo_batch_encode_steps(None, None, 1) == 1
    assert lib.ribo_batch_set_tile_modes(None, None, 0) == 1
    assert lib.ribo_batch_size(None) == 0
    lib.ribo_batch_destroy(None)


def test_world_footprint_counts_every_buffer(rw):
    """The footprint is the sum of the world's buffers (restated here from the
    buffer list: env cells C, fluid cells F, light cells L, multigrid M)."""
    for (gw, gh), (fw, fh), mg in (((2048, 2048), (2048, 2048), 16), ((256, 128), (128, 64), 8), ((96, 96), (96, 96), 8)):
        C, F, L = gw * gh, fw * fh, (gw // 2) * (gh // 2)
        M, nx, ny = 0, fw, fh
        while True:
            M += (nx * ny + 63) // 64 * 64
            if nx > mg and ny > mg and nx % 2 == 0 and ny % 2 == 0:
                nx, ny = nx // 2, ny // 2
            else:
                break
        terrain = 2 * C + 36 * ((gw + 2) // 3) * ((gh + 2) // 3) + 64
        tmaps = 128  # TMA descriptor of the stencil passes
        want = C * 48 + terrain + 24 * L + F * 101 + (fw + fh) * 4 + 96 + 64 * 48 + 16 + M * 14 + 2 * 64 * 464 + tmaps
        assert rw.world_footprint((gw, gh), (fw, fh), mg_min_size=mg) == want


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_server_without_gpu_reports_cuda_error(rw):
    with pytest.raises(rw.RiboError) as e:
        rw.Server(1 << 30)
    assert "CUDA_ERROR" in str(e.value)


def test_server_bad_arguments(rw):
    lib = rw.load_library()
    h = ctypes.c_void_p()
    cfg = rw.ServerCfg(0, 0, 0, 0, 1 << 30)  # max_chunk_steps 0
    assert lib.ribo_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    cfg = rw.ServerCfg(0, 8, 0, 0, 0)  # zero budget
    assert lib.ribo_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert lib.ribo_server_submit(None, None, None) == 1
    assert lib.ribo_server_iterate(None, None) == 1
    lib.ribo_server_destroy(None)


def test_reference_arm_runs_without_the_cuda_library(ro):
    """bench.py --impl reference times the CPU restatement alone: its process
    maps the oracle's library and never the product's (its SimParams come
    from the oracle's own table of the reference defaults)."""
    import json
    import sys

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "64",
                          "--steps", "3", "--warmup", "3", "--reference-seconds", "1"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    libs = line["native_libraries"]
    assert any("libribo_oracle" in p for p in libs), libs
    assert not any("libribo_world" in p for p in libs), libs
