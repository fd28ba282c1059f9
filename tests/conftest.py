import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    """The built C-ABI library (GPU tests only; it is the product)."""
    from adscf_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        from adscf_gb300 import build
        build.build()
    return _lib.load()


@pytest.fixture
def rng():
    return np.random.default_rng(1234)
