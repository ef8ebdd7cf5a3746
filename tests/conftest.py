"""Shared test setup: repo root on sys.path, the `gpu` marker, fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device for GPU tests.  A GPU test run without a GPU fails
    (it is never skipped silently)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from fluxvortex_gb300 import _capi
    _capi.load()
    return torch.device("cuda:0")


def rel_err(a, b):
    """max|a-b| / max|b|: the reference's own tolerance convention
    (tests/test_correctness.py:53-54 of the reference)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / (np.max(np.abs(b)) + 1e-300)) if b.size else 0.0
