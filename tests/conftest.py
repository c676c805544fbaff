"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o

    o.lib()
    return o


@pytest.fixture(scope="session")
def ctx():
    from crender_gb300 import api

    c = api.Context(0)
    yield c
    c.close()
