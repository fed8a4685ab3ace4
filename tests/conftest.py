import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


def random_fields(n, seed, so=True, coulomb=False):
    """Seeded smooth random fields for parity tests: f > 0, arbitrary grad f
    (not the gradient of f on purpose: H's terms are independent inputs)."""
    rng = np.random.default_rng(seed)
    ns = n ** 3
    f = 20.7 * (0.7 + 0.3 * rng.random(ns))
    gradf = rng.normal(0, 3.0, 3 * ns)
    U = -60 * rng.random(ns)
    W = rng.normal(0, 5.0, 3 * ns) if so else None
    UC = 10 * rng.random(ns) if coulomb else None
    return f, gradf, U, W, UC


def random_block(N, ncols, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(N, ncols)) + 1j * rng.normal(size=(N, ncols))
    return np.asfortranarray(X)
