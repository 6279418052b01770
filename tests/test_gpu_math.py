"""The constitutive kernel's own device math (dgx_device_math) against IEEE results:
the Newton-Raphson reciprocal within one ulp of the correctly rounded 1/x (exact where
it falls back to the division), x^(9/4) and x^19 within a few ulps of numpy's power, and
the mixed form's integer-pipe FP32 conversions bit-exact against a numpy restatement."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dm():
    from solver_cpp_gb300 import build, dgx
    build.build()
    L = dgx.lib()

    def run(fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty_like(x)
        dp = C.POINTER(C.c_double)
        dgx.check(L.dgx_device_math(fn, x.size, x.ctypes.data_as(dp), out.ctypes.data_as(dp)), "dgx_device_math")
        return out
    return run


def ulps(a, b):
    ia = a.view(np.int64).astype(object)
    ib = b.view(np.int64).astype(object)
    return np.array([abs(p - q) for p, q in zip(ia, ib)])


def test_reciprocal(dm):
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(0.5, 2.0, 20000), 10.0 ** rng.uniform(-290, 290, 20000),
                        -(10.0 ** rng.uniform(-30, 30, 5000)), 2.0 ** np.arange(-990, 990, 7.0),
                        np.nextafter(2.0 ** np.arange(-60, 60.0), 0.0), [1.0, -1.0, 3.0, 7.0, 1e8, 2.5e7]])
    r = dm(0, x)
    assert ulps(r, 1.0 / x).max() <= 1
    edge = np.array([0.0, -0.0, 1e-310, -5e-320, 1e305, -1e308, np.inf, -np.inf, np.nan])
    re = dm(0, edge)
    with np.errstate(divide="ignore", over="ignore"):
        ref = 1.0 / edge
    assert np.array_equal(re[:-1], ref[:-1]) and np.isnan(re[-1])
    assert np.signbit(re[1]) and not np.signbit(re[0])


def test_powers(dm):
    rng = np.random.default_rng(6)
    y = np.concatenate([rng.uniform(1e-6, 1.0, 20000), 10.0 ** rng.uniform(-25, 0, 5000)])
    assert np.max(np.abs(dm(1, y) / y ** 2.25 - 1.0)) < 1e-12
    x = rng.uniform(0.0, 1.5, 20000)
    p = dm(2, x)
    ref = x ** 19
    assert np.max(np.abs(p - ref) / np.maximum(ref, 1e-300)) < 1e-14


def f32_toward_zero(x):
    """FP64 -> FP32 rounded toward zero, FP32 subnormals flushed to signed zero, values
    beyond FP32 range to signed inf, NaN kept (numpy restatement of the device's to_f32)."""
    with np.errstate(over="ignore", invalid="ignore"):
        f = x.astype(np.float32)
        over = np.abs(f.astype(np.float64)) > np.abs(x)
        f = np.where(over & np.isfinite(x), np.nextafter(f, np.float32(0)), f)
        f = np.where(np.isfinite(x) & (np.abs(x) >= 2.0 ** 128), np.copysign(np.float32(np.inf), x), f)
        f = np.where(np.abs(f) < np.finfo(np.float32).tiny, np.copysign(np.float32(0), x), f)
    return f.astype(np.float64)


def test_integer_pipe_conversions(dm):
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-2.0, 2.0, 20000), 10.0 ** rng.uniform(-37, 38, 20000),
                        -(10.0 ** rng.uniform(-37, 38, 5000)), 2.0 ** np.arange(-126, 128.0),
                        np.nextafter(2.0 ** np.arange(-126, 128.0), 0.0),
                        [0.0, -0.0, 1e-40, -1e-45, 1e-300, 3.5e38, -1e39, 1e300, np.inf, -np.inf]])
    got = dm(3, x)
    ref = f32_toward_zero(x)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))
    assert np.isnan(dm(3, np.array([np.nan]))[0])


def hi_word_f32(x):
    """The mixed form's tolerance-scale conversion restated in numpy: the FP64 value with
    its low 32 bits cleared (20 mantissa bits, exact in FP32), signed zero below the FP32
    normal range, signed infinity above it and for NaN."""
    bits = x.view(np.uint64)
    e = (bits >> np.uint64(52)) & np.uint64(0x7ff)
    cut = (bits & np.uint64(0xffffffff00000000)).view(np.float64)
    with np.errstate(invalid="ignore"):
        sign = np.where(np.signbit(x), -1.0, 1.0)
    return np.where(e <= 896, sign * 0.0, np.where(e >= 1151, sign * np.inf, cut))


def test_tolerance_scale_conversion(dm):
    rng = np.random.default_rng(8)
    x = np.concatenate([rng.uniform(2.5e7, 7e7, 20000), 10.0 ** rng.uniform(-37, 38, 20000),
                        -(10.0 ** rng.uniform(-37, 38, 5000)), 2.0 ** np.arange(-126, 128.0),
                        np.nextafter(2.0 ** np.arange(-126, 128.0), 0.0),
                        [0.0, -0.0, 1e-40, -1e-45, 1e-300, 3.5e38, -1e39, 1e300, np.inf, -np.inf, np.nan]])
    got = dm(4, x)
    ref = hi_word_f32(x)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))
    fin = np.isfinite(x) & (np.abs(x) >= np.finfo(np.float32).tiny) & (np.abs(x) < 2.0 ** 128)
    assert np.max(np.abs(got[fin] - x[fin]) / np.abs(x[fin])) < 2.0 ** -20
