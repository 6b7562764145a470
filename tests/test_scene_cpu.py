"""Scene files (the reference's .ribo container, src/world/snapshot.rs):
the LZ4 block coder and the SimParams names, without a GPU."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_param_names():
    h = open(os.path.join(ROOT, "include", "ribo_world.h")).read()
    body = h[h.index("typedef struct ribo_sim_params"):h.index("} ribo_sim_params;")]
    return [n for _, n in re.findall(r"^\s*(float|uint32_t|int32_t)\s+([a-z_0-9]+)\s*;", body, re.M)]


def test_param_names_follow_the_struct(rw):
    names = rw.sim_param_names()
    assert names == header_param_names()
    assert names == [f[0] for f in rw.SimParams._fields_]
    assert len(names) == 116


def samples():
    rng = np.random.default_rng(5)
    yield b""
    yield b"x"
    yield b"abcdefghijkl"              # 12 bytes: no match allowed
    yield b"abcdabcdabcda"             # 13 bytes: the shortest input with a match
    yield bytes(100000)                # one long match
    yield bytes(rng.integers(0, 256, 70000, dtype=np.uint8))   # incompressible
    yield (b"0123456789" * 30000)[:299999]
    chem = rng.poisson(4, size=(64, 64, 4)).astype(np.uint32)  # a chem grid: small counts
    yield chem.tobytes()
    v = np.zeros((128, 128, 2), np.float32)
    v[40:80, 30:90] = rng.standard_normal((40, 60, 2)).astype(np.float32)
    yield v.tobytes()
    yield bytes(rng.integers(0, 4, 200000, dtype=np.uint8))    # long runs of 255-extended lengths


def test_lz4_round_trip(rw):
    for data in samples():
        block = rw.lz4_compress(data)
        assert len(block) <= len(data) + len(data) // 255 + 16
        assert rw.lz4_decompress(block, len(data)) == data


def test_lz4_blocks_are_standard(rw):
    """Blocks interoperate with an independent LZ4 block codec (the format the
    reference's lz4_flex writes after its 4-byte length)."""
    pa = pytest.importorskip("pyarrow")
    for data in samples():
        if not data:
            continue
        ours = rw.lz4_compress(data)
        assert pa.decompress(ours, decompressed_size=len(data), codec="lz4_raw", asbytes=True) == data
        theirs = pa.compress(data, codec="lz4_raw", asbytes=True)
        assert rw.lz4_decompress(theirs, len(data)) == data


def test_lz4_rejects_malformed_blocks(rw):
    data = (b"abcdefgh" * 1000)
    block = rw.lz4_compress(data)
    with pytest.raises(rw.RiboError):
        rw.lz4_decompress(block[: len(block) // 2], len(data))   # truncated
    with pytest.raises(rw.RiboError):
        rw.lz4_decompress(block, len(data) - 1)                  # output too small
    with pytest.raises(rw.RiboError):
        rw.lz4_decompress(bytes([0x0F, 0x01, 0x00]), 100)        # match before any output
