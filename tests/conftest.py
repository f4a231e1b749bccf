"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def sb(torch_cuda):
    """One SB_Handle per session on the current torch stream, as portBLAS's
    tests cache one queue per process (test/blas_test.hpp:96-100)."""
    from portblas_gb300 import build
    build.build()
    from portblas_gb300.blas import SB_Handle
    h = SB_Handle()
    yield h
    h.close()
