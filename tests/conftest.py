import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def rel_l1(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-field relative L1 error sum|a-b| / sum|b| over the first axis.

    Fields that are identically zero in b use the absolute L1 instead."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    num = np.abs(a - b).sum(axis=1)
    den = np.abs(b).sum(axis=1)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), num)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
