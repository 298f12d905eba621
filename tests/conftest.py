import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def W():
    """The product package with its library built in-tree."""
    from woodenpbrengine_gb300.build import build_library

    build_library()
    import woodenpbrengine_gb300 as W

    W.lib()
    return W


@pytest.fixture(scope="session")
def O():
    """The oracle binding (test infrastructure)."""
    from oracle.build import build_oracle

    build_oracle()
    from oracle import binding

    binding.lib()
    return binding


@pytest.fixture(scope="session")
def ctx(W):
    """A GPU context; GPU tests fail (not skip) when there is no device."""
    c = W.Context(0)
    yield c
    c.close()
