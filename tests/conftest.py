import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the CUDA library")


@pytest.fixture(scope="session")
def gpu_lib():
    """The device library, built in-tree; fails loudly when it cannot be built or loaded."""
    from magla_gb300 import build
    build.build_all()
    from magla_gb300 import _native
    return _native.gpu()


def build_vector(n, seed):
    """Seeded uniform[-1, 1) right-hand side (the reference's BuildVector distribution)."""
    return np.random.default_rng(seed).uniform(-1.0, 1.0, n)


def relative_residual(matrix, b, x):
    import oracle
    nb = float(np.sqrt(np.sum(np.asarray(b) ** 2)))
    r = oracle.residual_norm(matrix, b, x)
    return r / nb if nb > 0 else r


def max_relative_difference(actual, expected):
    scale = max(1e-300, float(np.max(np.abs(expected)))) if len(expected) else 1.0
    return float(np.max(np.abs(np.asarray(actual) - np.asarray(expected))) / scale) if len(expected) else 0.0
