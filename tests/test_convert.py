"""The stage kernel's FP32 <-> FP64 conversions run on the integer pipes
(a rounding by one 64-bit addition, a widening by shifts); they must agree
bit for bit with the hardware conversions on every input class: the normal
binary32 range, exact ties and their neighbours, the overflow and underflow
edges, subnormals, signed zeros, infinities and NaNs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs():
    rng = np.random.default_rng(7)
    n = 1 << 20
    # doubles across and beyond the binary32 exponent range
    x = np.ldexp(1.0 + rng.random(n), rng.integers(-170, 170, n)) * rng.choice([-1.0, 1.0], n)
    # exact round-to-nearest ties on the 29 dropped bits, and one unit either side
    t = rng.integers(0, 1 << 63, n, dtype=np.uint64)
    t = (t & ~np.uint64(0x1FFFFFFF)) | np.uint64(0x10000000)
    ties = np.concatenate([t, t + np.uint64(1), t - np.uint64(1)]).view(np.float64)
    # arbitrary bit patterns (their low words are arbitrary floats too)
    raw = rng.integers(0, np.iinfo(np.uint64).max, n, dtype=np.uint64, endpoint=True).view(np.float64)
    f32max = float(np.finfo(np.float32).max)
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan,
                      f32max, np.nextafter(f32max, np.inf), f32max * (1 + 2.0 ** -24), -f32max * (1 + 2.0 ** -24),
                      f32max * (1 + 2.0 ** -24 - 2.0 ** -40), 2.0 ** 128, 2.0 ** -126, -(2.0 ** -126),
                      2.0 ** -126 * (1 - 2.0 ** -25), 2.0 ** -127, 2.0 ** -149, 2.0 ** -150, 2.0 ** -151,
                      5e-324, 1e-300, 1e300, 1.0, -1.0, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24])
    return np.ascontiguousarray(np.concatenate([x, ties, raw, edges]))


def test_integer_conversions_equal_hardware(sgdg):
    x = _inputs()
    bad, first = ctypes.c_int64(), ctypes.c_int64()
    code = sgdg.lib().sgdg_selftest_convert(x, x.size, ctypes.byref(bad), ctypes.byref(first))
    assert code == 0
    assert bad.value == 0, "first mismatch at x = %r" % (x[first.value],)


def test_convert_selftest_empty(sgdg):
    bad, first = ctypes.c_int64(7), ctypes.c_int64(7)
    x = np.zeros(1)
    assert sgdg.lib().sgdg_selftest_convert(x, 0, ctypes.byref(bad), ctypes.byref(first)) == 0
    assert bad.value == 0 and first.value == -1
