import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _build():
    from alsvinn_gb300 import _build as b
    b.build_oracle()
    b.build_cuda()


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    _build()


@pytest.fixture(scope="session")
def cuda_device():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")


def interior(U, n, g):
    """Interior cells of padded arrays U[var, total] as [var, nz, ny, nx]."""
    dim = 3 if n[2] > 1 else (2 if n[1] > 1 else 1)
    t = [n[d] + 2 * g if d < dim else n[d] for d in range(3)]
    V = U.reshape(U.shape[0], t[2], t[1], t[0])
    gz, gy, gx = (g if dim > 2 else 0), (g if dim > 1 else 0), g
    return V[:, gz:gz + n[2], gy:gy + n[1], gx:gx + n[0]]


def rel_l1(a, b):
    """Per-variable relative L1 error sum|a-b| / sum|b|."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    den = np.abs(b).sum(axis=1)
    den[den == 0] = 1.0
    return np.abs(a - b).sum(axis=1) / den


def state_l1(a, b):
    """Per-variable L1 error for the FP32 state against the FP64 reference:
    sum|a-b| over max(sum|b| of the variable, sum|b| of variable 0, the
    density or u). A variable that starts at zero (a transverse momentum) is
    measured against the density's scale, the others against their own."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    den = np.maximum(np.abs(b).sum(axis=1), np.abs(b[0]).sum())
    return np.abs(a - b).sum(axis=1) / den
