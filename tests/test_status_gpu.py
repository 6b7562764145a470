"""Error path of the kernels' bounded waits, without a GPU fault.

Kernels never trap: a wait that gives up (a TMA copy that never completed)
sets a bit in the world's status word and returns.  Here the host half is
driven by writing the word between steps, and the device half by a
one-CTA kernel whose mbarrier wait runs out because nothing completes the
phase; the context keeps working after both."""
import ctypes

import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu

RIBO_TIMEOUT = 4
ERR_TIMEOUT = 1


def test_status_word_reports_timeout_once(rw):
    lib = rw.load_library()
    w = rw.World(64, seed=5, mg_min_size=16, mg_pre=3, mg_post=3)
    w.seed_inputs(synth.make_world_inputs(64, seed=5))
    w.encode_steps(2)
    w.sync()
    assert lib.ribo_world_raise_status(w._h, ERR_TIMEOUT) == 0
    assert lib.ribo_world_sync(w._h) == RIBO_TIMEOUT
    assert b"timed out" in lib.ribo_last_error()
    # the word was cleared: the world keeps stepping and conserves matter
    assert lib.ribo_world_sync(w._h) == 0
    before = w.ledger_blocking().total()
    w.encode_steps(2)
    w.sync()
    assert w.ledger_blocking().total() == before
    w.close()


def test_bounded_wait_runs_out_and_context_survives(rw):
    lib = rw.load_library()
    bits = ctypes.c_uint32(0)
    assert lib.ribo_selftest_bounded_wait(0, 1000, ctypes.byref(bits)) == 0
    assert bits.value == ERR_TIMEOUT
    # the device still runs a world step after the wait gave up
    w = rw.World(64, seed=6)
    w.seed_inputs(synth.make_world_inputs(64, seed=6))
    w.encode_steps(1)
    w.sync()
    assert np.all(np.isfinite(w.read(rw.VELOCITY)))
    w.close()
