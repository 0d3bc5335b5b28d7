"""The integer-arithmetic double <-> float conversions of the kernels (``xk_d2f``, ``xk_f2d`` in
``csrc/xk_common.cuh``), restated with NumPy integer operations: the same bits as the IEEE conversions
(round to nearest, ties to even; exact widening) for random values over the whole exponent range, exact
ties, zeros of both signs and the special values that the routines hand to the conversion instruction.
The GPU test ``test_conversions_in_integer_arithmetic_are_ieee`` checks the CUDA routines themselves."""

from __future__ import annotations

import numpy as np

U32 = np.uint32


def d2f(x):
    b = np.asarray(x, np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(U32)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(U32)
    e = (hi >> U32(20)) & U32(0x7FF)
    normal = (e - U32(897)) <= U32(253)  # the unsigned wrap of the CUDA test
    m = ((hi & U32(0xFFFFF)) << U32(3)) | (lo >> U32(29))
    r = lo & U32(0x1FFFFFFF)
    up = (r > U32(0x10000000)) | ((r == U32(0x10000000)) & ((m & U32(1)) == U32(1)))
    f = ((hi & U32(0x80000000)) | ((e - U32(896)) << U32(23)) | m) + up.astype(U32)
    out = f.view(np.float32).copy()
    zero = ((hi & U32(0x7FFFFFFF)) | lo) == 0
    out[zero] = (hi[zero] & U32(0x80000000)).view(np.float32)
    other = ~normal & ~zero  # the conversion instruction
    with np.errstate(over="ignore"):
        out[other] = np.asarray(x, np.float64)[other].astype(np.float32)
    return out


def f2d(v):
    f = np.asarray(v, np.float32).view(U32)
    e = (f >> U32(23)) & U32(0xFF)
    normal = (e - U32(1)) <= U32(253)
    hi = (f & U32(0x80000000)) | ((e + U32(896)) << U32(20)) | ((f & U32(0x7FFFFF)) >> U32(3))
    lo = f << U32(29)
    out = ((hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)).view(np.float64).copy()
    zero = (f & U32(0x7FFFFFFF)) == 0
    out[zero] = (f[zero].astype(np.uint64) << np.uint64(32)).view(np.float64)
    other = ~normal & ~zero
    out[other] = np.asarray(v, np.float32)[other].astype(np.float64)
    return out


def _same(a, b):
    """The same bits, NaNs (of any payload) aside, which must be NaN in both."""
    ua = a.view(np.uint32 if a.dtype == np.float32 else np.uint64)
    ub = b.view(np.uint32 if b.dtype == np.float32 else np.uint64)
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(nan_a, nan_b) and np.array_equal(ua[~nan_a], ub[~nan_b]))


def test_double_to_float_is_round_to_nearest_even():
    rng = np.random.default_rng(0)
    n = 1_000_000
    x = rng.standard_normal(n) * 10.0 ** rng.uniform(-45.0, 40.0, n)
    f = (rng.standard_normal(n) * 10.0 ** rng.uniform(-30.0, 30.0, n)).astype(np.float32)
    ties = f.astype(np.float64) + 0.5 * np.spacing(f).astype(np.float64)  # exactly half an ulp above
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-310, -1e-310, 3.4028235677973366e38,
                        3.4028235e38 * 1.0000001, 1.1754943508222875e-38, 1.1754942e-38, 2.0 ** -149, 5e-324])
    for arr in (x, ties, special):
        with np.errstate(over="ignore"):
            assert _same(d2f(arr), arr.astype(np.float32))


def test_float_to_double_is_exact():
    rng = np.random.default_rng(1)
    v = np.concatenate([(rng.standard_normal(1_000_000) * 10.0 ** rng.uniform(-38.0, 38.0, 1_000_000)).astype(np.float32),
                        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-40, 3.4028235e38], np.float32)])
    assert _same(f2d(v), v.astype(np.float64))
