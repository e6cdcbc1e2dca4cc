"""Shared fixtures.  `gpu` marks tests that need a GB300; everything else runs on CPU."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    from unsflow2d_gb300 import build
    build.build()
    import oracle
    oracle.lib()
    yield


def rel_err(gpu: np.ndarray, ref: np.ndarray) -> float:
    """Max-norm error relative to the field's own max magnitude (per last axis column)."""
    g = np.asarray(gpu, dtype=np.float64).reshape(len(gpu), -1)
    r = np.asarray(ref, dtype=np.float64).reshape(len(ref), -1)
    scale = np.maximum(np.abs(r).max(axis=0), 1e-300)
    return float((np.abs(g - r).max(axis=0) / scale).max())


@pytest.fixture
def assert_close():
    def _check(name, gpu, ref, rtol):
        e = rel_err(gpu, ref)
        assert np.all(np.isfinite(gpu)), f"{name}: non-finite GPU values"
        assert e <= rtol, f"{name}: relative max-norm error {e:.3e} > {rtol:.1e}"
        return e
    return _check
