"""Shared test setup: builds the native libraries once per session and
registers the `gpu` marker (tests that need a CUDA device)."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def native_built():
    from oracle import build as obuild
    from pascal_btdma_gb300 import build as pbuild

    obuild.build()
    pbuild.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def per_system_relerr(m, nsys, nrow, x, ref):
    """max over systems of max|x - ref| / max|ref| (reference GPU layout)."""
    x = np.asarray(x).reshape(m, nrow, nsys)
    r = np.asarray(ref).reshape(m, nrow, nsys)
    num = np.abs(x - r).max(axis=(0, 1))
    den = np.abs(r).max(axis=(0, 1))
    den = np.where(den == 0, 1.0, den)
    return float((num / den).max())
