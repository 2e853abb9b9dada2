import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libedgb300.so")


@pytest.fixture(scope="session")
def edlib():
    """The built library; built on demand (nvcc cross-compiles without a GPU)."""
    from hamiltonian_diagonalization_gb300.build import build
    build()
    from hamiltonian_diagonalization_gb300 import _capi
    return _capi.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda(edlib):
    """torch on cuda:0 with the engine's library loaded; fails loudly if absent."""
    import torch
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    assert edlib.ed_device_count() >= 1
    torch.cuda.init()
    return torch
