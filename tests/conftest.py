"""Shared test set-up: the 'gpu' marker, the in-tree build and import paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mpm3d-f90_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_addoption(parser):
    parser.addoption("--reference-tree", default=None,
                     help="MPM3D-F90 source tree (its Data/ and VolumetricLockingEx/ decks) for the tests "
                          "that read the reference's own files; default: $MPM3D_REFERENCE, else a "
                          "'reference' directory beside this repository")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def reference_tree_path(config=None):
    """The reference source tree, or None when it is not on this machine."""
    cand = [config.getoption("--reference-tree") if config is not None else None,
            os.environ.get("MPM3D_REFERENCE"),
            os.path.join(os.path.dirname(ROOT), "reference")]
    for c in cand:
        if c and os.path.isdir(os.path.join(c, "Data")):
            return c
    return None


@pytest.fixture(scope="session")
def reference_tree(request):
    """Path of the reference tree; tests that read it skip where it is absent
    (it is never needed by the GPU tests, whose decks are regenerated)."""
    p = reference_tree_path(request.config)
    if p is None:
        pytest.skip("reference tree not present (set MPM3D_REFERENCE or --reference-tree)")
    return p


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
