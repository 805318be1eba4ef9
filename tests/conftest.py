"""Shared test setup: the `gpu` marker, path setup and native builds."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C ABI)")


@pytest.fixture(scope="session")
def native():
    """Builds (if stale) and loads libyas_gb300, the generator and the oracle."""
    import __graft_entry__

    __graft_entry__.build()
    from yetanotherslam_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def cuda(native):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but CUDA is not available")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
