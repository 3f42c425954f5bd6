import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def rel_err_vec(a, b):
    """Per-particle vector-norm relative difference |a-b|/|b|."""
    num = np.linalg.norm(a - b, axis=1)
    den = np.linalg.norm(b, axis=1)
    return num / np.where(den > 0, den, 1.0)


@pytest.fixture(scope="session")
def gpu():
    import rebound_gb300
    rebound_gb300.load()
    return rebound_gb300
