"""Shared fixtures: import paths, the gpu marker, helpers to compare runs."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, 'acme-ecp_gb300'), os.path.join(REPO, 'oracle'), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (GB300)')


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope='session')
def gpu_lib():
    """The CUDA library, built in-tree; fails loudly when absent."""
    if not has_gpu():
        pytest.fail('gpu test selected but no CUDA device is visible')
    from crm_gb300 import build, lib
    build.build()
    return lib.load()


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    if den == 0.0:
        return 0.0 if num == 0.0 else np.inf
    return num / den
