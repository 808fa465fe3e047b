"""Shared fixtures.  The FP64 CPU oracle (oracle/) is the parity checker; it
is built here with make if needed.  GPU tests are marked ``gpu``."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    from rbc3d_gb300.abi import Library
    path = os.path.join(ROOT, "oracle", "liboracle_rbc3d.so")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s"], check=True)
    return Library(path, "rbc3d_oracle_")


@pytest.fixture(scope="session")
def gpu():
    """The product library.  No fallback: a missing build or a missing GPU fails."""
    from rbc3d_gb300 import build, library
    build.build()
    return library()
