"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; the rest run
on CPU only."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    return O.port()


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(GOLDEN, "ref_outputs.npz"))


@pytest.fixture(scope="session")
def ans1024():
    return np.load(os.path.join(GOLDEN, "ans1024.npy"))


@pytest.fixture(scope="session")
def nstab():
    return np.load(os.path.join(GOLDEN, "nstab.npz"))


@pytest.fixture(scope="session")
def lib():
    """The solver library (built in-tree on first use)."""
    import tpr_gb300
    return tpr_gb300.load()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
