"""Shared test set-up: the 'gpu' marker, the in-tree build and import paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mpm3d-f90_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Compile the library and the oracle once per session (no-op if current)."""
    import build  # mpm3d-f90_gb300/build.py

    build.build_all()
    return True


@pytest.fixture(scope="session")
def oracle_mod(built):
    import oracle as o

    return o


@pytest.fixture(scope="session")
def gpu_mod(built):
    import mpm3d_gb300 as m

    return m
