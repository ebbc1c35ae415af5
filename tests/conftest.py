import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs through the C-ABI")
    config.addinivalue_line("markers", "slow: full-size parity case (minutes of oracle time)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    if not os.path.exists(O.LIB_PATH):
        O.build()
    return O


@pytest.fixture(scope="session")
def ng():
    """The product package with its native library loaded (fails loudly if not built)."""
    import numcosmo_gb300 as ng
    from numcosmo_gb300 import _lib

    _lib.load(build_if_missing=True)
    return ng


@pytest.fixture(scope="session")
def gpu(ng):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible")
    return ng


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0
