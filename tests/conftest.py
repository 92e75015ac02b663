import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native library")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def orc():
    from oracle.loader import oracle
    return oracle()


@pytest.fixture(scope="session")
def gpu_lib():
    """The native library; GPU tests fail loudly if it cannot be built or
    loaded (no silent fallback)."""
    import molsim_gb300
    molsim_gb300.build()
    return molsim_gb300.abi.load_library()
