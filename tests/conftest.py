import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import binding

    binding.lib()
    return binding


@pytest.fixture(scope="session")
def gpu_lib():
    from stormbird_gb300 import build as sb_build

    sb_build.build()
    from stormbird_gb300.native import lib

    return lib()
