"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/ribo_oracle.cpp into oracle/_build/libribo_oracle.so with
plain IEEE single-precision semantics: no FMA contraction and no fast-math,
so the oracle's float results do not depend on the host ISA (x86-64 or
aarch64).  The reference itself (Rust + WGSL through wgpu) cannot be built
here, so there is no oracle/_ref.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ribo_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libribo_oracle.so")
DEPS = [
    SRC,
    os.path.join(HERE, "..", "include", "ribo_world.h"),
    os.path.join(HERE, "..", "ribossome-v2_gb300", "csrc", "ribo_fmath.h"),
]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(OUT):
        t = os.path.getmtime(OUT)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return OUT
    cmd = [
        "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing",
        "-Wall", "-Wno-unused-function",
        SRC, "-o", OUT + ".tmp",
    ]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
