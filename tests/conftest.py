import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


def maxrel(a, b) -> float:
    """max |a - b| / max |b| -- the error measure of the reference's GPU tests."""
    a, b = np.asarray(a), np.asarray(b)
    den = float(np.max(np.abs(b))) if b.size else 0.0
    num = float(np.max(np.abs(a - b))) if a.size else 0.0
    return num / den if den > 0 else num


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def native():
    """Build (if stale) and load the native library and module; GPU tests only."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diaq_gb300 import build

    build.build()
    from diaq_gb300 import capi, diaq_gpu

    capi.lib()
    return capi, diaq_gpu
