import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
PKG = ROOT / "fortkernels-_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


def rel_err(a, b):
    """Elementwise |a - b| / |b| for complex arrays."""
    a = np.asarray(a)
    b = np.asarray(b)
    return np.abs(a - b) / np.maximum(np.abs(b), np.finfo(float).tiny)


def normwise_err(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="session")
def sigma_lib():
    """The CUDA library; GPU tests fail (not skip) when it cannot load."""
    import sigma_gb300
    import torch

    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    sigma_gb300.load()
    return sigma_gb300
