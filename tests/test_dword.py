"""CPU checks of the double-word (FP32 pair) arithmetic of the mixed update
(csrc/dword.cuh): the split of a double into a nearest float and a float
residual, and the FP32 face state (Sigma, l, Pi) whose pressure recovery
Pi = (E - |r x l|^2 / (2 Sigma)) (gam - 1) is evaluated in double-word
arithmetic instead of FP64.  Exact rational arithmetic is the reference;
the recovered pressure must be the exact value rounded to FP32 within one
ulp, down to kinetic energies within 1e-5 of the total energy."""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
CSRC = REPO / "muscl-scheme-on-spherical-mesh-wip_gb300" / "csrc"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("dword") / "libdword.so"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", f"-I{CSRC}",
           f"-I{REPO / 'include'}", str(REPO / "tests" / "cpp" / "dword.cpp"), "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True)
    return ctypes.CDLL(str(out))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _split(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    h = np.empty(x.shape, np.float32)
    lo = np.empty(x.shape, np.float32)
    lib.dw_split(_p(x), _p(h), _p(lo), ctypes.c_int64(x.size))
    return h, lo


def _face_state(lib, u, r, gam_m1):
    u = np.ascontiguousarray(u, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    w = np.empty(u.shape, np.float32)
    lib.dw_face_state(_p(u), _p(r), ctypes.c_double(gam_m1), _p(w), ctypes.c_int64(len(u)))
    return w


def _ulps(a, b):
    """Distance in FP32 ulps between positive float32 arrays."""
    return np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))


def test_split_nearest_and_residual(lib):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(20000) * np.exp(rng.uniform(-60, 60, 20000))
    x = np.concatenate([x, [1.0, -1.0, 2.0 - 2.0 ** -40, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24,
                            np.nextafter(1.0, 2.0), 3.4e38, -1e-30]])
    h, lo = _split(lib, x)
    assert np.array_equal(h, x.astype(np.float32))
    err = np.abs((h.astype(np.float64) - x) + lo.astype(np.float64))
    assert np.all(err <= np.abs(x) * 2.0 ** -47)
    # |l| is at most half an FP32 ulp of h
    assert np.all(np.abs(lo) <= np.spacing(np.abs(h)) / 2)


def test_split_outside_float_range(lib):
    x = np.array([0.0, -0.0, 1e-300, -1e-40, 1e39, -1e300, np.inf, -np.inf, np.nan])
    h, lo = _split(lib, x)
    assert np.all(lo == 0)
    assert np.array_equal(h[:2].view(np.uint32), np.array([0.0, -0.0], np.float32).view(np.uint32))
    assert h[2] == 0 and h[3] == 0 and np.signbit(h[3])
    assert np.isposinf(h[4]) and np.isneginf(h[5]) and np.isposinf(h[6]) and np.isneginf(h[7])
    assert np.isnan(h[8])


def _exact_pressure(u, r, gam_m1):
    sg, lx, ly, lz, E = (Fraction(float(v)) for v in u)
    rx, ry, rz = (Fraction(float(v)) for v in r)
    cx, cy, cz = ry * lz - rz * ly, rz * lx - rx * lz, rx * ly - ry * lx
    p = (E - (cx * cx + cy * cy + cz * cz) / (2 * sg)) * Fraction(gam_m1)
    return max(p, Fraction(1e-16))


@pytest.mark.parametrize("ratio", [10.0, 1.0, 1e-2, 1e-4, 1e-5])
def test_pressure_within_one_ulp(lib, ratio):
    """Pi / (gam - 1) = ratio * KE: the smaller the ratio, the stronger the
    cancellation in E - KE."""
    rng = np.random.default_rng(7 + int(round(abs(np.log10(ratio)) * 10)))
    n = 400
    r = rng.standard_normal((n, 3))
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    sg = np.exp(rng.uniform(np.log(1e-6), np.log(10.0), n))
    v = rng.standard_normal((n, 3)) * np.exp(rng.uniform(-3, 2, (n, 1)))
    l = sg[:, None] * np.cross(r, v)
    l += rng.standard_normal((n, 3)) * 1e-3 * np.abs(l).max(axis=1, keepdims=True)  # a radial part
    gam_m1 = 1.0 / 3.0
    ke = np.einsum("ij,ij->i", np.cross(r, l), np.cross(r, l)) / (2 * sg)
    E = ke * (1 + ratio)
    u = np.column_stack([sg, l, E])
    w = _face_state(lib, u, r, gam_m1)
    assert np.array_equal(w[:, :4], u[:, :4].astype(np.float32))
    exact = np.array([np.float32(float(_exact_pressure(u[i], r[i], gam_m1))) for i in range(n)])
    ulps = _ulps(w[:, 4], exact)
    assert ulps.max() <= 1, (ratio, ulps.max())
    # the FP64 evaluation of the same formula, rounded to FP32, for comparison
    c = np.cross(r, l)
    p64 = np.maximum((E - 0.5 * np.einsum("ij,ij->i", c, c) / sg) * gam_m1, 1e-16).astype(np.float32)
    assert (_ulps(w[:, 4], p64) <= 1).all()
    if ratio >= 1e-2:
        assert np.mean(w[:, 4] == exact) > 0.99


def test_pressure_floor_and_nan(lib):
    r = np.array([[0.0, 0.0, 1.0]] * 3)
    u = np.array([[1.0, 1.0, 0.0, 0.0, 0.4],    # E < KE: floored
                  [1.0, 0.0, 0.0, 0.0, 0.0],    # zero pressure: floored
                  [1.0, np.nan, 0.0, 0.0, 1.0]])  # NaN: floored, like (1e-16 < p) ? p : 1e-16
    w = _face_state(lib, u, r, 0.5)
    assert np.all(w[:, 4] == np.float32(1e-16))
