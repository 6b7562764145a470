import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ribossome-v2_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def rw():
    """The product's Python mirror, with libribo_world.so built in-tree."""
    import build as pkg_build

    pkg_build.build()
    import ribo_world

    ribo_world.load_library()
    return ribo_world


@pytest.fixture(scope="session")
def ro():
    """The CPU oracle (test infrastructure)."""
    import ribo_oracle

    ribo_oracle.load()
    return ribo_oracle
