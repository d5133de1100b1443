"""Shared fixtures.  ``-m gpu`` tests need a CUDA device; everything else
runs on the CPU in a few minutes."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build(ref=True)
    return O


@pytest.fixture(scope="session")
def qgwlib():
    from qgw_gb300 import build, capi
    build.build()
    return capi
