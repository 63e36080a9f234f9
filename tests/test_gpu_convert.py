"""The FP32 face kernels widen their Gauss-quadrature sums to FP64 on the integer pipes
(f32_to_f64) before the FP64 S2O4 stage combination.  That conversion must equal the hardware
conversion bit for bit on every value the kernels produce: normal numbers of both signs and
every exponent, signed zeros, infinities and NaNs; FP32 subnormals, which the FP32 kernels flush
to zero, read as signed zero."""
import ctypes

import numpy as np
import pytest

from hos_gb300.solver import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


def _convert(x):
    lib = load()
    lib.hos_last_error.restype = ctypes.c_char_p
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.size, dtype=np.float64)
    rc = lib.hos_convert_selftest(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.c_size_t(x.size))
    assert rc == 0, lib.hos_last_error()
    return y


def test_normal_values_and_zeros_convert_exactly():
    rng = np.random.default_rng(7)
    # every exponent of the normal range, random mantissas, both signs; the extremes; zeros
    bits = rng.integers(0, 1 << 23, size=200_000, dtype=np.uint32)
    bits |= rng.integers(1, 255, size=bits.size, dtype=np.uint32) << 23
    bits |= rng.integers(0, 2, size=bits.size, dtype=np.uint32) << 31
    extra = np.array([0x00800000, 0x80800000, 0x7f7fffff, 0xff7fffff, 0x3f800000, 0, 0x80000000], dtype=np.uint32)
    x = np.concatenate([bits, extra]).view(np.float32)
    y = _convert(x)
    assert np.array_equal(y.view(np.uint64), x.astype(np.float64).view(np.uint64))


def test_special_values_keep_their_class():
    x = np.array([np.inf, -np.inf, np.nan, -np.nan], dtype=np.float32)
    sub = np.array([0x00000001, 0x007fffff, 0x80000001], dtype=np.uint32).view(np.float32)
    y = _convert(np.concatenate([x, sub]))
    assert y[0] == np.inf and y[1] == -np.inf
    assert np.isnan(y[2]) and np.isnan(y[3])
    assert np.array_equal(y[4:].view(np.uint64), np.array([0, 0, 1 << 63], dtype=np.uint64))
