"""Builds libribo_world.so (the CUDA world-step library) in-tree.

Every translation unit is compiled by nvcc for sm_103a only, in parallel,
then linked into _build/libribo_world.so next to this file.  Float
semantics are pinned: no FMA contraction (-fmad=false), IEEE division and
square root, no flush-to-zero, so kernel results match the CPU oracle bit
for bit.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libribo_world.so")
INCLUDE = os.path.join(HERE, "..", "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-Xptxas", "-warn-spills",
    "--expt-relaxed-constexpr",
]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


# The bounds-checked variant: kernels test their riskiest indices and record
# RIBO_ERR_BOUNDS in the world's status word instead of accessing out of
# range (ribo_world_sync then fails); a separate library for test runs.
CHECKED_DIR = os.path.join(OUT_DIR, "checked")
CHECKED_LIB = os.path.join(CHECKED_DIR, "libribo_world.so")
CHECKED_FLAGS = ("-DRB_BOUNDS_CHECK",)


def _compile(src: str, extra, out_dir: str, force: bool) -> str:
    obj = os.path.join(out_dir, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep and not force:
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
    subprocess.run(cmd, check=True)
    return obj


def build(verbose: bool = False, extra=(), checked: bool = False) -> str:
    """Builds the library (or, with checked=True, the bounds-checked variant
    in _build/checked/); extra flags force a rebuild of the default one."""
    out_dir, lib = (CHECKED_DIR, CHECKED_LIB) if checked else (OUT_DIR, LIB)
    flags = tuple(extra) + (CHECKED_FLAGS if checked else ())
    force = bool(extra)
    os.makedirs(out_dir, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, flags, out_dir, force), srcs))
    if os.path.exists(lib) and not force:
        t = os.path.getmtime(lib)
        if all(os.path.getmtime(o) <= t for o in objs):
            return lib
    cmd = [nvcc()] + ARCH + ["-shared", "-o", lib + ".tmp"] + objs
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    args = sys.argv[1:]
    if args[:1] == ["--checked"]:
        print(build(verbose=True, extra=args[1:], checked=True))
    else:
        print(build(verbose=True, extra=args))
