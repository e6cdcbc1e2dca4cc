"""The kernels' exact replacements for FP64 divisions (uns_phys.cuh):
division through a precomputed reciprocal with Markstein's correction must
equal IEEE division bit for bit, and the exact ratio comparison that picks
the smallest of several quotients must agree with exact rational
arithmetic, including ties."""
import ctypes as C
from fractions import Fraction

import numpy as np
import pytest

from unsflow2d_gb300 import abi

pytestmark = pytest.mark.gpu
D = C.POINTER(C.c_double)


def _lib():
    lib = abi.gpu_lib()
    lib.uns_selftest_div.argtypes = [D, D, D, C.c_int]
    lib.uns_selftest_ratio.argtypes = [D, D, D, D, C.POINTER(C.c_int), C.c_int]
    return lib


def _p(a):
    return a.ctypes.data_as(D)


def test_division_through_reciprocal_equals_ieee_division():
    rng = np.random.default_rng(5)
    n = 1 << 20
    a = rng.standard_normal(n) * np.exp2(rng.integers(-300, 300, n).astype(float))
    b = rng.standard_normal(n) * np.exp2(rng.integers(-300, 300, n).astype(float))
    # mantissas near powers of two and exact quotients, where rounding is delicate
    k = n // 8
    b[:k] = np.exp2(rng.integers(-40, 40, k).astype(float)) * (1.0 + rng.integers(0, 8, k) * 2.0 ** -52)
    a[k:2 * k] = b[k:2 * k] * rng.integers(1, 1000, k)
    special = np.array([0.0, -0.0, 1.0, -1.0, 3.0, np.finfo(float).max, np.finfo(float).tiny, 5e-324,
                        np.inf, -np.inf, np.nan, 1e-310, 1e300, 1e-300])
    a = np.concatenate([a, special, special[::-1]])
    b = np.concatenate([b, special[::-1], special])
    b[b == 0.0] = 1.0
    out = np.zeros_like(a)
    assert _lib().uns_selftest_div(_p(a), _p(b), _p(out), len(a)) == 0
    with np.errstate(all="ignore"):
        ref = a / b
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(out), nan)
    bad = np.flatnonzero((out.view(np.uint64) != ref.view(np.uint64)) & ~nan)
    assert len(bad) == 0, [(float(a[i]).hex(), float(b[i]).hex(), float(out[i]).hex(), float(ref[i]).hex())
                           for i in bad[:8]] + [len(bad)]


def test_exact_ratio_comparison():
    rng = np.random.default_rng(6)
    n = 20000
    a = np.abs(rng.standard_normal(n)) * np.exp2(rng.integers(-60, 20, n).astype(float))
    b = np.abs(rng.standard_normal(n)) * np.exp2(rng.integers(-60, 20, n).astype(float)) + 1e-30
    c = a * (1.0 + rng.integers(-2, 3, n) * 2.0 ** -52)   # ratios within a few ulps of each other
    d = b.copy()
    m = n // 2
    c[m:] = np.abs(rng.standard_normal(n - m))
    d[m:] = np.abs(rng.standard_normal(n - m)) + 0.1
    t = n // 10  # exact ties: c/d == a/b with c = 2a, d = 2b
    c[:t], d[:t] = 2 * a[:t], 2 * b[:t]
    a[-5:] = 0.0
    lt = np.zeros(n, dtype=np.int32)
    rc = _lib().uns_selftest_ratio(_p(a), _p(b), _p(c), _p(d), lt.ctypes.data_as(C.POINTER(C.c_int)), n)
    assert rc == 0
    applies = lt >= 0
    assert applies.mean() > 0.99
    exact = np.array([Fraction(x) / Fraction(y) < Fraction(z) / Fraction(w) for x, y, z, w in zip(a, b, c, d)])
    assert np.array_equal(lt[applies].astype(bool), exact[applies])

