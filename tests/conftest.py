"""Shared pytest set-up: the `gpu` marker, and import paths for the oracle (the
checker) and the product package (whose directory name is not a Python identifier)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbca.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gbca():
    """The product package, loaded from its directory."""
    import __graft_entry__ as ge
    return ge.load_package()
