"""The allocation-free pressure solve (ribo_pressure_solve_noalloc).

It serves callers that cannot allocate device memory while they run -- a
host that reserves its whole device budget at start-up, or a frame loop that
cannot absorb the synchronisation cudaMalloc/cudaFree may cause -- by keeping
the multigrid hierarchy in a fixed array inside the library.  Here it is
called through the C ABI on caller-owned buffers and must reproduce, bit for
bit, the pressure the world step's own (allocating) solve produced from the
same divergence, wall mask and warm start, on two calls in a row.  This file
is collected last so a failure here cannot hide the results of other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(rw):
    lib = rw.load_library()
    fn = lib.ribo_pressure_solve_noalloc
    fn.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + \
        [ctypes.c_uint32] * 5 + [ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return lib, fn


# (fluid width, height): the square the limit allows, a level-0 grid small
# enough for the single-CTA coarse kernel to take whole (it then reads the
# caller's wall mask, divergence and pressure directly), a rectangle, a grid
# whose halving stops early at odd sides (90 x 66 -> 45 x 33), and the
# largest grid the scratch holds.
GRIDS = [(256, 256), (64, 64), (96, 160), (90, 66), (512, 512)]


@pytest.mark.parametrize("grid", GRIDS, ids=[f"{w}x{h}" for w, h in GRIDS])
def test_noalloc_pressure_solve_matches_world_step(rw, grid):
    import torch

    import synth

    lib, fn = _entry(rw)
    nw, nh = grid
    w = rw.World(grid, seed=5, mg_min_size=16, mg_pre=3, mg_post=3)
    w.seed_inputs(synth.make_world_inputs(grid, seed=5))
    w.params.dt = 1.0
    w.params.transport_every = 1
    w.params.sun_heat = 0.0
    w.settings.fluid_substep = 1
    w.settings.mg_cycles = 2
    w.encode_steps(1)  # a non-zero warm start
    for call in range(2):
        p0 = w.read(rw.PRESSURE).copy()
        w.encode_steps(1)
        div = w.read(rw.DIVERGENCE)
        mask = w.read(rw.SOLID_MASK)
        p1 = w.read(rw.PRESSURE)
        t_div = torch.from_numpy(np.ascontiguousarray(div)).cuda()
        t_mask = torch.from_numpy(np.ascontiguousarray(mask).view(np.int32)).cuda()
        t_p = torch.from_numpy(p0).cuda()
        torch.cuda.synchronize()
        st = fn(nw, nh, t_div.data_ptr(), t_mask.data_ptr(), t_p.data_ptr(), 16, 3, 3, 30, 2, None)
        assert st == 0, lib.ribo_last_error()
        torch.cuda.synchronize()
        got = t_p.cpu().numpy()
        diff = np.nonzero(got.view(np.uint32) != p1.view(np.uint32))[0]
        assert diff.size == 0, f"{nw}x{nh} call {call}: {diff.size} cells differ, first {diff[:3]}"
    w.close()


def test_noalloc_rejects_grids_above_the_scratch_limit(rw):
    import torch

    lib, fn = _entry(rw)
    t = torch.zeros(8, device="cuda")
    st = fn(1024, 1024, t.data_ptr(), t.data_ptr(), t.data_ptr(), 0, 0, 0, 0, 0, None)
    assert st == 1
    assert b"512x512" in lib.ribo_last_error()
