"""CPU checks of the integer FP32 <-> FP64 conversions the mixed update uses
instead of FP64-pipe conversions (csrc/fp_convert.cuh): float -> double is
exact; double -> float rounds to nearest even, flushes results below the
smallest FP32 normal to a signed zero, overflows to infinity and keeps NaN.
numpy's conversions (IEEE round to nearest even, with subnormals) are the
reference; only the subnormal range differs, by the flush."""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
CSRC = REPO / "muscl-scheme-on-spherical-mesh-wip_gb300" / "csrc"
FMIN = np.finfo(np.float32).tiny


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("fpconv") / "libfpconv.so"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{CSRC}", f"-I{REPO / 'include'}",
           str(REPO / "tests" / "cpp" / "fp_convert.cpp"), "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True)
    return ctypes.CDLL(str(out))


def _d2f(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(x.shape, np.float32)
    lib.conv_d2f(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(x.size))
    return y


def _f2d(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape, np.float64)
    lib.conv_f2d(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(x.size))
    return y


def _expected_d2f(x):
    with np.errstate(over="ignore"):
        y = x.astype(np.float32)
    small = np.abs(y) < FMIN
    y[small] = np.copysign(np.float32(0), x[small]).astype(np.float32)
    return y


def _same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nan = np.isnan(a) & np.isnan(b)
    return np.array_equal(a.view(np.uint32 if a.dtype == np.float32 else np.uint64)[~nan],
                          b.view(np.uint32 if b.dtype == np.float32 else np.uint64)[~nan]) and \
        np.array_equal(np.isnan(a), np.isnan(b))


def test_double_to_float_random_bits(lib):
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2 ** 64, size=2_000_000, dtype=np.uint64)
    x = bits.view(np.float64)
    assert _same_bits(_d2f(lib, x), _expected_d2f(x))


def test_double_to_float_state_range_and_ties(lib):
    rng = np.random.default_rng(1)
    x = rng.normal(size=1_000_000) * 10.0 ** rng.uniform(-30, 30, size=1_000_000)
    # exact ties at the FP32 rounding point: mantissa bit 28 set, bits below clear
    f = rng.normal(size=100_000).astype(np.float32)
    ties = f.astype(np.float64).view(np.uint64) | np.uint64(1 << 28)
    x = np.concatenate([x, ties.view(np.float64)])
    # around the ends of the FP32 range
    edge = np.array([np.finfo(np.float32).max, float(np.finfo(np.float32).max) * (1 + 2 ** -25),
                     float(np.finfo(np.float32).max) * (1 + 2 ** -23), 2.0 ** 128, FMIN, FMIN * 0.75,
                     FMIN * (1 - 2 ** -30), 0.0, -0.0, np.inf, -np.inf, np.nan, 1e-8, 1e20, 1e40])
    x = np.concatenate([x, edge, -edge])
    assert _same_bits(_d2f(lib, x), _expected_d2f(x))


def test_float_to_double_is_exact(lib):
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 2 ** 32, size=2_000_000, dtype=np.uint64).astype(np.uint32)
    f = bits.view(np.float32)
    with np.errstate(invalid="ignore"):
        expect = f.astype(np.float64)
    sub = (np.abs(f) < FMIN) & (f != 0)
    expect[sub] = np.copysign(0.0, f[sub].astype(np.float64))
    assert _same_bits(_f2d(lib, f), expect)
    assert _same_bits(_f2d(lib, np.array([np.inf, -np.inf, 0.0, -0.0], np.float32)),
                      np.array([np.inf, -np.inf, 0.0, -0.0]))


def test_nan_test_from_bits(lib):
    x = np.array([np.nan, -np.nan, np.inf, -np.inf, 0.0, 1.0, -1e300,
                  np.uint64(0x7ff0000000000001).view(np.float64), np.uint64(0xfff8000000000000).view(np.float64)])
    y = np.empty(x.size, np.int32)
    lib.conv_isnan(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(x.size))
    assert np.array_equal(y.astype(bool), np.isnan(x))
