"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA kernels through the C ABI)")


@pytest.fixture(scope="session")
def pbf():
    import __graft_entry__

    return __graft_entry__.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    return o


@pytest.fixture(scope="session")
def cuda(pbf):
    """Skip-free GPU guard: a gpu-marked test on a machine without CUDA fails loudly."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)
