import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import py_oracle
    py_oracle.lib()
    return py_oracle


@pytest.fixture(scope="session")
def native_lib():
    from fuzzyblue_gb300 import build
    build.build()
    from fuzzyblue_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def builder(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    from fuzzyblue_gb300.api import Builder
    b = Builder(0)
    yield b
    b.close()
