"""CPU checks of the hand-written local adjoints (adjoint_rev.cuh).

The per-slot Riemann flux reverse, the per-face reconstruction reverse, the
source-term and pressure-conversion reverses are compiled for the host
(tests/cpp/adjoint_local.cpp, g++ -ffp-contract=off) and checked against
the forward-mode duals of the same code (full Jacobians, dot products) and
against central finite differences of the plain double evaluation.
"""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
CSRC = REPO / "muscl-scheme-on-spherical-mesh-wip_gb300" / "csrc"
GAM = 1.25
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_D)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("adjlocal") / "libadjlocal.so"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wno-unknown-pragmas",
           f"-I{CSRC}", f"-I{REPO / 'include'}", str(REPO / "tests" / "cpp" / "adjoint_local.cpp"), "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True)
    return ctypes.CDLL(str(out))


def _state(rng, r, speed):
    sig = rng.uniform(0.5, 2.0)
    pi = rng.uniform(0.5, 2.0)
    t = rng.normal(size=3)
    t -= t.dot(r) * r
    v = t / np.linalg.norm(t) * speed
    return np.array([sig, *(sig * np.cross(r, v)), pi / (GAM - 1) + sig * v.dot(v) / 2])


def _slot_geom(rng):
    ec = rng.normal(size=3)
    ec *= 0.999 / np.linalg.norm(ec)
    en = rng.normal(size=3)
    en -= en.dot(ec) / ec.dot(ec) * ec
    en /= np.linalg.norm(en)
    ecn = np.linalg.norm(ec)
    return np.array([*ec, ecn, *en, *np.cross(en, ec / ecn)]), ec / ecn


def _flux(lib, uL, uR, g, solver):
    F, Jf, Jr = np.zeros(5), np.zeros(50), np.zeros(50)
    mism = lib.adj_flux_jac(_p(uL), _p(uR), _p(g), ctypes.c_double(GAM), solver, _p(F), _p(Jf), _p(Jr))
    return mism, F, Jf.reshape(5, 10), Jr.reshape(5, 10)


@pytest.mark.parametrize("solver", [1, 2, 3])
def test_flux_reverse_matches_dual_jacobian(lib, solver):
    rng = np.random.default_rng(10 + solver)
    kinds = {"left": 0, "right": 0, "both": 0}
    for _ in range(600):
        g, r = _slot_geom(rng)
        sp = rng.choice([0.01, 0.5, 1.5, 3.0])
        uL, uR = _state(rng, r, sp * rng.uniform(0, 1)), _state(rng, r, sp * rng.uniform(0, 1))
        mism, _, Jf, Jr = _flux(lib, uL, uR, g, solver)
        assert mism == 0, "dual values differ from the double evaluation"
        assert np.abs(Jf - Jr).max() <= 1e-12 * np.abs(Jf).max()
        left, right = np.abs(Jf[:, :5]).max() > 0, np.abs(Jf[:, 5:]).max() > 0
        kinds["both" if left and right else ("left" if left else "right")] += 1
    # the random set reaches the upwind sides and the star / averaged states
    assert all(v > 0 for v in kinds.values()), kinds


@pytest.mark.parametrize("solver", [1, 2, 3])
def test_flux_dual_jacobian_matches_finite_differences(lib, solver):
    rng = np.random.default_rng(20 + solver)
    for _ in range(60):
        g, r = _slot_geom(rng)
        uL, uR = _state(rng, r, rng.uniform(0, 2)), _state(rng, r, rng.uniform(0, 2))
        _, _, J, _ = _flux(lib, uL, uR, g, solver)
        x = np.concatenate([uL, uR])
        Jfd = np.zeros((5, 10))
        for j in range(10):
            h = 1e-6 * max(1.0, abs(x[j]))
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            Jfd[:, j] = (_flux(lib, xp[:5], xp[5:], g, solver)[1] - _flux(lib, xm[:5], xm[5:], g, solver)[1]) / (2 * h)
        assert np.abs(Jfd - J).max() <= 1e-6 * np.abs(J).max()


@pytest.mark.parametrize("mode", ["generic", "flat_field", "zero_forward_difference"])
def test_recon_reverse_dot_product(lib, mode):
    """<upb, J v> (recon_face on Dual<1>) == <J^T upb, v> (recon_face_rev + beta scatter)."""
    rng = np.random.default_rng({"generic": 1, "flat_field": 2, "zero_forward_difference": 3}[mode])
    for _ in range(300):
        n = int(rng.choice([5, 6]))
        nf = 1 + 4 * n
        sten = np.arange(1, nf, dtype=np.int32).reshape(n, 4).T.copy()
        beta = rng.uniform(0.2, 0.8, size=(4, n))
        hpm = rng.uniform(0.5, 1.5, size=(2, n)) * 0.01
        bm = rng.uniform(0.5, 1.5, size=(1, n)) * 0.01
        eta = np.vstack([hpm[0] / bm[0], hpm[1] / bm[0]])
        arc = rng.uniform(30, 90, size=(1, n))
        ec = rng.normal(size=(3, n))
        ec *= 0.9995 / np.linalg.norm(ec, axis=0)
        en = rng.normal(size=(3, n))
        en -= (en * ec).sum(0) / (ec * ec).sum(0) * ec
        en /= np.linalg.norm(en, axis=0)
        ecn = np.linalg.norm(ec, axis=0)[None]
        W = np.empty((5, nf))
        W[0] = 1 + 0.3 * rng.uniform(-1, 1, nf)
        W[1:4] = 0.3 * rng.uniform(-1, 1, (3, nf))
        W[4] = 1 + 0.3 * rng.uniform(-1, 1, nf)
        if mode == "flat_field":  # pp = pm = 0: NaN ratio, limiter 0
            W[2, :] = 0.1
        if mode == "zero_forward_difference":  # pp = 0, pm != 0: infinite ratio
            for j in range(n):
                W[3, sten[0, j]] = W[3, 0]
                W[3, sten[1, j]] = W[3, 0]
        V = rng.normal(size=(5, nf))
        upb = rng.normal(size=(5, n))
        out, up = np.zeros(2), np.zeros((5, n))
        mism = lib.adj_recon_dot(n, nf, sten.ctypes.data_as(_I), _p(beta), _p(hpm), _p(bm), _p(eta), _p(arc), _p(ec),
                                 _p(ecn), _p(en), ctypes.c_double(GAM), ctypes.c_double(5e-4), _p(W), _p(V), _p(upb),
                                 _p(out), _p(up))
        assert mism == 0, "dual values differ from the double evaluation"
        assert np.isfinite(out).all()
        assert abs(out[0] - out[1]) <= 1e-10 * abs(out[0])


@pytest.mark.parametrize("friction_on", [0, 1])
def test_source_reverse_matches_finite_differences(lib, friction_on):
    rng = np.random.default_rng(30 + friction_on)
    for _ in range(100):
        r = rng.normal(size=3)
        r /= np.linalg.norm(r)
        t = rng.normal(size=3)
        t -= t.dot(r) * r
        v = t * rng.uniform(0, 0.5)
        sig, pi = rng.uniform(0.5, 2), rng.uniform(0.5, 2)
        w = np.array([sig, *(sig * np.cross(r, v)), pi])
        prm = np.array([rng.uniform(0, 0.1), rng.uniform(-.5, .5), rng.uniform(-.5, .5), rng.uniform(1e-3, 1e-1),
                        rng.uniform(5, 20)])
        phys = np.array([GAM, rng.uniform(0, 0.3), 0.5, rng.choice([1e-6, 1e-2])])
        J = np.zeros(50)
        lib.adj_source_jac(_p(w), _p(r), _p(prm), _p(phys), friction_on, _p(J))
        J = J.reshape(5, 10)

        def ev(x):
            res = np.zeros(5)
            lib.adj_source_eval(_p(x[:5].copy()), _p(r), _p(x[5:].copy()), _p(phys), friction_on, _p(res))
            return res

        x = np.concatenate([w, prm])
        Jfd = np.zeros((5, 10))
        for j in range(10):
            h = 1e-6 * max(1e-2, abs(x[j]))
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            Jfd[:, j] = (ev(xp) - ev(xm)) / (2 * h)
        assert np.abs(J - Jfd).max() <= 1e-6 * np.abs(J).max()


def test_pressure_conversion_reverse_matches_finite_differences(lib):
    rng = np.random.default_rng(40)
    for _ in range(100):
        r = rng.normal(size=3)
        r /= np.linalg.norm(r)
        u = np.array([rng.uniform(.5, 2), *rng.uniform(-.5, .5, 3), rng.uniform(2, 8)])
        w, J = np.zeros(5), np.zeros(25)
        lib.adj_prim(_p(u), _p(r), ctypes.c_double(GAM), _p(w), _p(J))
        J = J.reshape(5, 5)
        Jfd = np.zeros((5, 5))
        for j in range(5):
            h = 1e-6 * max(1, abs(u[j]))
            up, um = u.copy(), u.copy()
            up[j] += h
            um[j] -= h
            wp, wm, scratch = np.zeros(5), np.zeros(5), np.zeros(25)
            lib.adj_prim(_p(up), _p(r), ctypes.c_double(GAM), _p(wp), _p(scratch))
            lib.adj_prim(_p(um), _p(r), ctypes.c_double(GAM), _p(wm), _p(scratch))
            Jfd[:, j] = (wp - wm) / (2 * h)
        assert np.abs(J - Jfd).max() <= 1e-6 * np.abs(J).max()
