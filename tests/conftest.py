"""Shared pytest configuration: the `gpu` marker and library build fixtures."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native library")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the oracle and the native library once per session (nvcc cross-compiles
    without a GPU)."""
    import oracle_lib
    from parthenon_gb300 import build
    oracle_lib.build()
    build.build()
    yield


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
