"""The fp32 elementary functions the tessellation kernel and the oracle share
(rive-runtime_gb300/csrc/rive_fp32_math.h), measured against double-precision
libm over dense sweeps. Errors are in units in the last place (ulp) of the
fp32 result, with an absolute floor of 2^-24 near zero crossings. Bounds:
sin/cos 2 ulp on |x| <= 64 (angles the tessellation forms stay within a few
turns), acos 2 ulp on [-1, 1], cube root 2 ulp on (0, 3.4e38]."""
import ctypes

import numpy as np
import pytest

import oracle


def _eval(fn, x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib = oracle.lib()
    lib.oracle_math_eval.restype = ctypes.c_int
    rc = lib.oracle_math_eval(ctypes.c_int(fn), x.ctypes.data_as(ctypes.c_void_p),
                              out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(x.size))
    assert rc == 0
    return out


def _ulp_err(got, want):
    w32 = want.astype(np.float32)
    spacing = np.maximum(np.spacing(np.abs(w32)).astype(np.float64), 2.0 ** -24)
    return np.abs(got.astype(np.float64) - want) / spacing


def test_sin_cos_within_2ulp():
    x = np.concatenate([np.linspace(-64, 64, 2_000_001, dtype=np.float32),
                        np.linspace(-1e-3, 1e-3, 20_001, dtype=np.float32)])
    x64 = x.astype(np.float64)
    es = _ulp_err(_eval(0, x), np.sin(x64))
    ec = _ulp_err(_eval(1, x), np.cos(x64))
    assert es.max() <= 2.0, float(es.max())
    assert ec.max() <= 2.0, float(ec.max())


def test_acos_within_2ulp_and_exact_ends():
    x = np.concatenate([np.linspace(-1, 1, 4_000_001, dtype=np.float32),
                        1 - np.arange(0, 5000, dtype=np.float32) * np.float32(2 ** -24),
                        -1 + np.arange(0, 5000, dtype=np.float32) * np.float32(2 ** -24)])
    got = _eval(2, x)
    e = _ulp_err(got, np.arccos(x.astype(np.float64)))
    assert e.max() <= 2.0, (float(e.max()), float(x[np.argmax(e)]))
    assert _eval(2, np.float32([1.0]))[0] == 0.0
    assert np.isnan(_eval(2, np.float32([1.5, -1.0001, np.nan]))).all()


def test_cbrt_within_2ulp():
    rng = np.random.default_rng(3)
    bits = rng.integers(1, 0x7f7fffff, 2_000_000, dtype=np.uint32)
    x = np.concatenate([bits.view(np.float32), np.linspace(1e-6, 1e3, 100_001, dtype=np.float32),
                        np.float32([1e-45, 1.1754942e-38, 8.0, 27.0, 1.0])])
    got = _eval(3, x)
    e = _ulp_err(got, np.cbrt(x.astype(np.float64)))
    assert e.max() <= 2.0, (float(e.max()), float(x[np.argmax(e)]))
    assert _eval(3, np.float32([0.0]))[0] == 0.0
    assert np.isinf(_eval(3, np.float32([np.inf]))[0])


@pytest.mark.parametrize("fn", [0, 1])
def test_sin_cos_propagate_nan_and_inf(fn):
    assert np.isnan(_eval(fn, np.float32([np.nan, np.inf, -np.inf]))).all()
