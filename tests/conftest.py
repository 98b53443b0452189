import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "3d_droplet_simulation_2007_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdsg.so")


def pkg():
    return importlib.import_module(PKG_NAME)


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def dsg():
    return pkg()


@pytest.fixture(scope="session")
def gpu_lib():
    if not has_gpu():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    m = pkg()
    m.build.build()
    return m


def relerr(x, ref):
    """max|x-ref| / max|ref| (norm-relative, 0 when both vanish)."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    scale = np.max(np.abs(ref)) if ref.size else 0.0
    diff = np.max(np.abs(x - ref)) if ref.size else 0.0
    if scale == 0.0:
        return float(diff)
    return float(diff / scale)


def interior(a):
    return a[1:-1, 1:-1, 1:-1]
