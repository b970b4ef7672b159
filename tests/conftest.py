import importlib
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
def oracle():
    import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def dccm():
    """The product package (ctypes mirror of the C ABI); the library must be built."""
    m = importlib.import_module("dennou-ccm_gb300")
    m.load()
    return m


@pytest.fixture(scope="session")
def synth():
    return importlib.import_module("dennou-ccm_gb300.synth")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch


def rel_l2(a, b):
    """Relative L2 error of a against b (complex arrays as real pairs)."""
    a, b = np.asarray(a), np.asarray(b)
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        a = np.ascontiguousarray(a, np.complex128).view(np.float64)
        b = np.ascontiguousarray(b, np.complex128).view(np.float64)
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)
