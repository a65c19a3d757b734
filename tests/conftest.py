import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(ROOT / "tests" / "golden" / "golden.npz"))


@pytest.fixture(scope="session")
def golden_confocal():
    """The reference test's own fixture at full size: 20 confocal frames of 256 x 256, lags 1..9."""
    return dict(np.load(ROOT / "tests" / "golden" / "golden_confocal.npz"))


def gpu_ready() -> bool:
    try:
        import torch
    except ImportError:
        return False
    return torch.cuda.is_available()


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and load the sm_103a library; GPU tests fail loudly without it."""
    from fastddm_gb300 import _build, _lib

    _build.build()
    return _lib.load()
