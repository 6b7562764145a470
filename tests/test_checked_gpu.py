"""The bounds-checked build (-DRB_BOUNDS_CHECK): the kernels test their
riskiest indices -- the transport scatter's window bins, accumulator slots,
far-destination atomics and mover queue, the fused fluid passes' box
indices -- and record an error instead of accessing out of range.  Small
parity cases run on it in a child process (the library is loaded once per
process) and must stay bit-exact with the oracle with no check firing."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_parity():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "ribossome-v2_gb300"))
    import build

    build.build(checked=True)
    out = subprocess.run([sys.executable, os.path.join(HERE, "checked_run.py")], capture_output=True, text=True,
                         timeout=900)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout[-2000:] + out.stderr[-4000:]
