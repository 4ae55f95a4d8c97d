"""pytest set-up: the `gpu` marker, import paths, one build of every library per session."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(REPO, "vulkan-restir-pt_gb300")
for p in (PKG_DIR, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def ref_available():
    from oracle import pyoracle
    return os.path.exists(pyoracle.REF_LIB)
