"""Shared pytest configuration: the `gpu` marker and repository imports."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libbcx.so")


@pytest.fixture(scope="session")
def cuda():
    """The torch module with CUDA initialised (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    torch.cuda.init()
    return torch
