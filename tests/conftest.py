"""pytest configuration: the `gpu` marker, import paths and in-tree builds."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(Path(__file__).resolve().parent)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (run on the GPU box)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (g++) and, when stale, the CUDA library (nvcc)."""
    import oracle

    oracle.build()
    from exoblas_gb300 import build as b

    b.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
