"""Test configuration: the `gpu` marker and shared helpers.

CPU tests (``-m "not gpu"``) check the oracle against its pins, the host
logic and the C-ABI exports; GPU tests compare the CUDA engine, called
through its C-ABI, with the oracle on the same seeded inputs.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def require_gpu():
    if not gpu_available():
        pytest.fail("GPU test run without a visible CUDA device")


def rel_err(a, b):
    """Norm-wise relative error max|a-b| / max|b| (0 if both are zero)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if a.size else 0.0
    return 0.0 if den == 0.0 and num == 0.0 else num / den
