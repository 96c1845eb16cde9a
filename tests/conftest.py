import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "isosurface-analysis_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def ctx():
    import isosim
    c = isosim.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def ref():
    import oracle
    r = oracle.load_reference()
    if r is None:
        pytest.skip("reference harness (oracle/_ref) not built here")
    return r
