import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """Build the in-tree CUDA library (nvcc cross-compiles without a GPU)."""
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def pkg(built_lib):
    return built_lib


@pytest.fixture(scope="session")
def orc():
    from oracle import scft_oracle
    return scft_oracle
