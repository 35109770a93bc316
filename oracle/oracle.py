"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker or the timed CPU
baseline, never as part of the product path.  See splash_oracle.cpp for the
reference functions it restates.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

_lib = None


def library() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing: run __graft_entry__.build()")
        lib = C.CDLL(str(LIB))
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        lib.oracle_create.restype = C.c_void_p
        lib.oracle_create.argtypes = [C.c_int, C.c_int, C.c_int, dp, ip, ip, ip, dp, dp, dp, dp, dp,
                                      dp, ip, ip, dp, dp, C.c_double, C.c_double, dp, C.c_int,
                                      C.c_double, C.c_double, C.c_int, dp, C.c_int, C.c_int]
        lib.oracle_destroy.argtypes = [C.c_void_p]
        lib.oracle_do_step.argtypes = [C.c_void_p, C.c_double]
        lib.oracle_do_step.restype = C.c_int
        lib.oracle_do_steps.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.oracle_do_steps.restype = C.c_int
        lib.oracle_get_state.argtypes = [C.c_void_p, dp]
        lib.oracle_set_state.argtypes = [C.c_void_p, dp]
        lib.oracle_info.argtypes = [C.c_void_p, dp]
        lib.oracle_get_uplus.argtypes = [C.c_void_p, dp]
        lib.oracle_flux_star.argtypes = [C.c_void_p, dp, dp, C.c_int, C.c_int, dp]
        lib.oracle_flux_star.restype = C.c_int
        lib.oracle_limiter.argtypes = [C.c_void_p, dp, dp, C.c_int, C.c_int, C.c_double, dp]
        lib.oracle_source.argtypes = [C.c_void_p, dp, C.c_int, dp]
        lib.oracle_iso_flux.argtypes = [C.c_void_p, dp, C.c_int, C.c_int, dp]
        lib.oracle_iso_char_vel.argtypes = [C.c_void_p, dp, dp, C.c_int, C.c_int, dp]
        _lib = lib
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Oracle:
    """One CPU restatement instance over a reference-numbered geometry.

    ``geom`` is a mapping with the arrays of geometry/MUSCL_geometry.hpp
    flattened per slot (splash_gb300.Geometry provides it) plus h0 and
    round_diff attributes/keys.
    """

    def __init__(self, geom, U_in, gam: float, omega_ns: float, accretion_on: bool,
                 params: list[float], solver: int, threads: int = 0, dim: int = 5):
        lib = library()
        g = geom
        self._keep = {k: (_d(g[k]) if np.asarray(g[k]).dtype.kind == "f" else _i(g[k]))
                      for k in ("vertices", "face_off", "face_vtx", "nbr_edge", "face_centers",
                                "area", "edge_normals", "bm_dist", "h_plus", "h_minus",
                                "ff_plus", "ff_minus", "beta_plus", "beta_minus")}
        k = self._keep
        self.nf = k["face_off"].shape[0] - 1
        self.ns = int(k["face_off"][-1])
        nv = k["vertices"].reshape(-1, 3).shape[0]
        self.dim = dim
        U = _d(U_in).reshape(self.nf, dim)
        P = _d(params)
        h0 = g.h0 if hasattr(g, "h0") else float(g["h0"])
        rd = g.round_diff if hasattr(g, "round_diff") else float(g["round_diff"])
        ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double if a.dtype == np.float64 else C.c_int))
        self.h = lib.oracle_create(nv, self.nf, self.ns, ptr(k["vertices"]), ptr(k["face_off"]),
                                   ptr(k["face_vtx"]), ptr(k["nbr_edge"]), ptr(k["face_centers"]),
                                   ptr(k["area"]), ptr(k["edge_normals"]), ptr(k["bm_dist"]),
                                   ptr(k["h_plus"]), ptr(k["h_minus"]), ptr(k["ff_plus"]),
                                   ptr(k["ff_minus"]), ptr(k["beta_plus"]), ptr(k["beta_minus"]),
                                   h0, rd, ptr(U), dim, gam, omega_ns, 1 if accretion_on else 0,
                                   ptr(P), solver, threads)
        if not self.h:
            raise RuntimeError("oracle_create rejected its arguments")
        self._lib = lib

    def __del__(self):
        if getattr(self, "h", None):
            self._lib.oracle_destroy(self.h)
            self.h = None

    def do_step(self, dt0: float) -> int:
        return self._lib.oracle_do_step(self.h, dt0)

    def do_steps(self, n: int, dt0: float) -> int:
        return self._lib.oracle_do_steps(self.h, n, dt0)

    def get_state(self) -> np.ndarray:
        U = np.empty((self.nf, self.dim))
        self._lib.oracle_get_state(self.h, U.ctypes.data_as(C.POINTER(C.c_double)))
        return U

    def set_state(self, U) -> None:
        U = _d(U)
        self._lib.oracle_set_state(self.h, U.ctypes.data_as(C.POINTER(C.c_double)))

    def info(self) -> dict:
        out = np.zeros(12)
        self._lib.oracle_info(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return {"t": out[0], "dt": out[1], "max_vel": out[2], "stop": bool(out[3]),
                "steps": int(out[4]), "area_coeff": out[5], "total_mass": out[6],
                "diag": out[7:12].copy()}

    def get_uplus(self) -> np.ndarray:
        out = np.empty((self.ns, self.dim))
        self._lib.oracle_get_uplus(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def flux_star(self, uL, uR, face: int, edge: int):
        F = np.empty(self.dim)
        dp = C.POINTER(C.c_double)
        bits = self._lib.oracle_flux_star(self.h, _d(uL).ctypes.data_as(dp), _d(uR).ctypes.data_as(dp),
                                          face, edge, F.ctypes.data_as(dp))
        return F, bits

    def limiter(self, r, w, face: int, edge: int, dt_member: float) -> np.ndarray:
        out = np.empty(self.dim)
        dp = C.POINTER(C.c_double)
        self._lib.oracle_limiter(self.h, _d(r).ctypes.data_as(dp), _d(w).ctypes.data_as(dp),
                                 face, edge, dt_member, out.ctypes.data_as(dp))
        return out

    def source(self, u, face: int) -> np.ndarray:
        out = np.empty(self.dim)
        dp = C.POINTER(C.c_double)
        self._lib.oracle_source(self.h, _d(u).ctypes.data_as(dp), face, out.ctypes.data_as(dp))
        return out

    # isothermal solver (solver 4, dim 4)
    def iso_flux(self, u, face: int, edge: int) -> np.ndarray:
        out = np.empty(4)
        dp = C.POINTER(C.c_double)
        self._lib.oracle_iso_flux(self.h, _d(u).ctypes.data_as(dp), face, edge, out.ctypes.data_as(dp))
        return out

    def iso_char_vel(self, uL, uR, face: int, edge: int) -> np.ndarray:
        out = np.empty(2)
        dp = C.POINTER(C.c_double)
        self._lib.oracle_iso_char_vel(self.h, _d(uL).ctypes.data_as(dp), _d(uR).ctypes.data_as(dp), face, edge,
                                      out.ctypes.data_as(dp))
        return out
