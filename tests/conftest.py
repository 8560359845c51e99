"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; the rest run on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libqslc.so")


@pytest.fixture(scope="session")
def port():
    """The oracle (CPU restatement), built on first use."""
    import oracle
    oracle.build(reference=False)
    return oracle


@pytest.fixture(scope="session")
def qsl():
    """The CUDA backend; fails loudly when the library or the device is missing."""
    import qsl_gb300
    qsl_gb300.build.build() if not os.path.exists(qsl_gb300.LIB_PATH) else None
    return qsl_gb300


def random_state(rng, n, dtype=np.complex128):
    v = rng.uniform(-1, 1, 1 << n) + 1j * rng.uniform(-1, 1, 1 << n)
    v /= np.linalg.norm(v)
    return v.astype(dtype)


def random_np_state(rng, n, w, dtype=np.complex128):
    import oracle
    v = np.zeros(1 << n, dtype=np.complex128)
    idx = oracle.generate_lookup(n, w).astype(np.int64)
    v[idx] = rng.normal(size=idx.size) + 1j * rng.normal(size=idx.size)
    v /= np.linalg.norm(v)
    return v.astype(dtype)


def bits(a: np.ndarray) -> np.ndarray:
    """Raw bits of a complex array, for bit-exact comparisons."""
    return a.view(np.uint64 if a.dtype == np.complex128 else np.uint32)
