"""Shared fixtures.  `gpu` marks tests that need a GB300; everything else runs on CPU.

Parity criteria used across the GPU tests (FP64):
  * fields (states, primitives, spectral radii, dt, norms): max-norm error
    <= rtol * max|field| per column;
  * residuals: |gpu - oracle| <= rtol * lambda_i * max|q_j| per entry -- a
    cell/node residual is a near-cancelling sum of face fluxes of that size,
    so its rounding error is bounded by the terms, not by the small sum;
  * gradients: |gpu - oracle| <= rtol * (max|grad col| + max|q_var| * inv_h),
    inv_h being the mesh's largest sum of gradient weights; where a field is
    uniform to rounding its gradient is pure rounding noise and only the
    second term is meaningful.
"""
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
    """Max-norm error relative to the field's own max magnitude (per column)."""
    g = np.asarray(gpu, dtype=np.float64).reshape(len(gpu), -1)
    r = np.asarray(ref, dtype=np.float64).reshape(len(ref), -1)
    scale = np.maximum(np.abs(r).max(axis=0), 1e-300)
    return float((np.abs(g - r).max(axis=0) / scale).max())


def res_err(gpu, ref, la, q) -> float:
    """Residual error relative to the flux scale lambda_i * max|q_j|."""
    scale = np.asarray(la)[:, None] * np.abs(np.asarray(q)).max(axis=0)[None, :4]
    return float((np.abs(np.asarray(gpu) - np.asarray(ref)) / np.maximum(scale, 1e-300)).max())


def grad_err(gpu, ref, q, inv_h) -> float:
    g = np.asarray(gpu).reshape(len(gpu), 4, 2)
    r = np.asarray(ref).reshape(len(ref), 4, 2)
    qmax = np.abs(np.asarray(q)[:, :4]).max(axis=0)  # per variable
    scale = np.abs(r).max(axis=0) + (qmax * inv_h)[:, None]
    return float((np.abs(g - r) / scale[None]).max())


def inv_h_cc(m) -> float:
    """Largest face-length sum over cell area (bounds GG / LSQ weight sums)."""
    per = np.zeros(m["noc"])
    np.add.at(per, m["fin"], m["farea"])
    inner = m["fout"] < m["noc"]
    np.add.at(per, m["fout"][inner], m["farea"][inner])
    return float((per / m["cv"]).max())


def inv_h_nc(m) -> float:
    w = np.hypot(m["wx"], m["wy"])
    s = np.add.reduceat(w, m["v2v_off"][:-1])
    return float(s.max())


@pytest.fixture
def assert_close():
    def _check(name, gpu, ref, rtol):
        e = rel_err(gpu, ref)
        assert np.all(np.isfinite(gpu)), f"{name}: non-finite GPU values"
        assert e <= rtol, f"{name}: relative max-norm error {e:.3e} > {rtol:.1e}"
        return e
    return _check
