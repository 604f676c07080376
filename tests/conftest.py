import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gmu-water-simulation_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running GPU case at full benchmark size")


@pytest.fixture(scope="session")
def sphlib():
    """The built C-ABI library (built in-tree on first use; never a CPU fallback)."""
    import sph_build  # gmu-water-simulation_gb300/sph_build.py

    sph_build.build()
    import sphcuda

    return sphcuda


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.build()
    return oracle
