"""Test configuration: the ``gpu`` marker, import paths, and shared helpers."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "acoustic3d-fd_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if stale) and load the engine library."""
    import build as pkg_build
    pkg_build.build()
    import a3d
    return a3d.lib()
