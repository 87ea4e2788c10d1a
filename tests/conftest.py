"""Shared fixtures.  `-m "not gpu"` runs everywhere; `-m gpu` needs a GB300."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fringe-sgc_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build libfsgc and the oracle once per session if they are missing."""
    import build as fsgc_build  # fringe-sgc_gb300/build.py

    if not os.path.exists(fsgc_build.LIB):
        fsgc_build.build()
    if not os.path.exists(os.path.join(ORACLE, "_build", "liboracle.so")):
        subprocess.run(["make", "-s", "-C", ORACLE], check=True)


@pytest.fixture(scope="session")
def ctx(built):
    import fsgc

    c = fsgc.Context(0)
    yield c
    c.close()
