import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native parts once per session (no-op when up to date)."""
    from glemur_gb300 import _build
    from oracle import build as oracle_build
    _build.build_all()
    oracle_build.build_all()


def relerr(a, b):
    """max |a - b| / max |b| over the array."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def inner(a):
    return a[1:-1, 1:-1, 1:-1]


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
