"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` need a CUDA device and the built library; everything else
runs on the CPU (oracle checks, host logic, symbol exports).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built neon_gb300 library")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def ngb():
    import neon_gb300
    neon_gb300.build()
    neon_gb300.lib()
    return neon_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a CUDA device")
    return torch.device("cuda:0")
