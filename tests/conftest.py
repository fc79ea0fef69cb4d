"""Shared fixtures.  Markers: ``gpu`` (needs a CUDA device and the built
library).  Everything unmarked runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libfockgb300.so")


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from strawberryfields_gb300 import _lib

    _lib.load()  # fails loudly if the library was not built
    return torch.device("cuda", 0)


@pytest.fixture
def rng():
    return np.random.default_rng(1234)


def random_state(rng, shape, pure=True):
    """Random normalised ket, or random density matrix with interleaved axes."""
    if pure:
        x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        return x / np.linalg.norm(x)
    n = len(shape) // 2
    D = shape[0]
    k = rng.normal(size=(D,) * n + (3,)) + 1j * rng.normal(size=(D,) * n + (3,))
    flat = k.reshape(D ** n, 3)
    rho = flat @ flat.conj().T
    rho /= np.trace(rho)
    rho = rho.reshape((D,) * (2 * n))
    perm = []
    for i in range(n):
        perm += [i, n + i]
    return np.ascontiguousarray(np.transpose(rho, perm))
