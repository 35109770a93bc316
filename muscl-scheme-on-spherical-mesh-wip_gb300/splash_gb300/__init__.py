"""ctypes binding of the GB300 MUSCL step (``include/splash_gb300.h``).

The product is the C ABI in ``lib/libsplash_gb300.so``; this module is a thin
binding used by the test-suite, the benchmark and Python callers.  It mirrors
the reference's solver classes (``Riemann_solvers/HLLE_p.hpp``,
``HLLC.hpp``, ``HLLCplus.hpp``): same constructor arguments, ``do_step``,
``time``, ``get_stop_check`` and the ``write_t_*`` writers.

There is no fallback: if the shared library is missing or CUDA is
unavailable, construction raises.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import initial_conditions  # noqa: F401  (re-exported helper module)
from . import input_recipes  # noqa: F401  (the reference's make_input.py recipes)
from . import workloads  # noqa: F401  (seeded synthetic workloads)

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "lib" / "libsplash_gb300.so"

MESH_ICOSPHERE_HEX = 0
MESH_QUAD_SPHERE = 1
MESH_ICOSPHERE = 2

SOLVER_HLLE_P = 1
SOLVER_HLLC = 2
SOLVER_HLLCPLUS = 3
SOLVER_HLLE = 4  # isothermal, dim 4

PREC_FP64 = 0
PREC_MIXED = 1

STOP_NAN_FLUX = 1
STOP_NAN_WAVESPEED = 2
STOP_WAVE_ORDER = 4
STOP_NEG_EXTRA_DT = 8

# every entry point declared in include/splash_gb300.h
EXPORTED = (
    "splash_last_error", "splash_version", "splash_create", "splash_destroy",
    "splash_do_step", "splash_do_steps", "splash_do_steps_host", "splash_synchronize", "splash_time",
    "splash_stop_check", "splash_error_word", "splash_last_dt", "splash_steps",
    "splash_n_faces", "splash_dim", "splash_get_state", "splash_set_state",
    "splash_diagnostics", "splash_get_permutation", "splash_write_t_rho",
    "splash_write_t_p", "splash_write_t_curl", "splash_write_t_omega_z",
    "splash_write_t_L", "splash_get_light_curves", "splash_write_final_state",
    "splash_geometry_build", "splash_geometry_free", "splash_geometry_info",
    "splash_geometry_get", "splash_stream", "splash_kernel_times", "splash_launch_times", "splash_memory",
    "splash_ensemble_create", "splash_ensemble_destroy", "splash_ensemble_do_steps",
    "splash_ensemble_synchronize", "splash_ensemble_stream", "splash_ensemble_get_state",
    "splash_ensemble_member_info", "splash_ensemble_schedule", "splash_ensemble_size",
    "splash_ensemble_set_schedule",
    "splash_cfl_dt_noalloc",
    "splash_adjoint_create", "splash_adjoint_destroy", "splash_adjoint_forward",
    "splash_adjoint_backward", "splash_adjoint_run", "splash_tlm_run", "splash_adjoint_info",
    "splash_adjoint_error_word", "splash_adjoint_dt_schedule", "splash_face_geometry",
    "splash_adjoint_branch_tape",
)


class SplashError(RuntimeError):
    """A C ABI call returned a non-zero status."""


class MeshDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("level", C.c_int),
        ("n_vertices", C.c_int), ("vertices", C.POINTER(C.c_double)),
        ("n_faces", C.c_int), ("face_offsets", C.POINTER(C.c_int)),
        ("face_vertices", C.POINTER(C.c_int)),
    ]


class Params(C.Structure):
    _fields_ = [
        ("accretion_rate", C.c_double), ("e_acc", C.c_double), ("omega_acc_abs", C.c_double),
        ("tilt_angle", C.c_double), ("acc_width", C.c_double), ("alpha", C.c_double),
        ("friction_on", C.c_int),
    ]


class Member(C.Structure):
    _fields_ = [
        ("mesh_kind", C.c_int), ("level", C.c_int), ("U_in", C.POINTER(C.c_double)),
        ("gam", C.c_double), ("omega_ns", C.c_double), ("accretion_on", C.c_int),
        ("params", Params), ("solver_kind", C.c_int),
    ]


_lib = None


def library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads (once) and returns the shared library; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path or os.environ.get("SPLASH_GB300_LIB", LIB_PATH))
    if not p.exists():
        raise SplashError(f"{p} not found: build it with __graft_entry__.build() "
                          f"(muscl-scheme-on-spherical-mesh-wip_gb300/build.py)")
    lib = C.CDLL(str(p))
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    vp = C.c_void_p
    lib.splash_last_error.restype = C.c_char_p
    lib.splash_version.restype = C.c_char_p
    lib.splash_create.argtypes = [C.POINTER(MeshDesc), dp, C.c_int, C.c_double, C.c_double, C.c_int,
                                  C.POINTER(Params), C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.POINTER(vp)]
    for name, args in {
        "splash_destroy": [vp], "splash_do_step": [vp, C.c_double],
        "splash_do_steps": [vp, C.c_int, C.c_double], "splash_synchronize": [vp],
        "splash_do_steps_host": [vp, dp, C.c_int, C.c_double, dp],
        "splash_time": [vp, dp], "splash_stop_check": [vp, ip],
        "splash_error_word": [vp, C.POINTER(C.c_uint32)], "splash_last_dt": [vp, dp],
        "splash_steps": [vp, C.POINTER(C.c_int64)], "splash_n_faces": [vp, ip],
        "splash_dim": [vp, ip], "splash_get_state": [vp, dp], "splash_set_state": [vp, dp],
        "splash_diagnostics": [vp, dp], "splash_get_permutation": [vp, ip],
        "splash_write_t_rho": [vp, C.c_char_p], "splash_write_t_p": [vp, C.c_char_p],
        "splash_write_t_curl": [vp, C.c_char_p], "splash_write_t_omega_z": [vp, C.c_char_p],
        "splash_write_t_L": [vp, C.c_char_p, C.c_char_p, C.c_char_p],
        "splash_get_light_curves": [vp, dp], "splash_write_final_state": [vp, C.c_char_p],
        "splash_geometry_build": [C.POINTER(MeshDesc), C.c_int, C.POINTER(vp)],
        "splash_geometry_free": [vp],
        "splash_geometry_info": [vp, C.POINTER(C.c_int64), dp],
        "splash_geometry_get": [vp, C.c_char_p, vp, C.c_size_t, C.POINTER(C.c_size_t)],
        "splash_stream": [vp, C.POINTER(vp)],
        "splash_kernel_times": [vp, C.c_int, C.c_double, dp],
        "splash_launch_times": [vp, C.c_int, C.c_double, dp, C.c_int, ip],
        "splash_memory": [vp, C.POINTER(C.c_int64)],
        "splash_ensemble_create": [C.POINTER(Member), C.c_int, C.c_int, C.c_int, C.POINTER(vp)],
        "splash_ensemble_destroy": [vp], "splash_ensemble_do_steps": [vp, C.c_int, C.c_double],
        "splash_ensemble_synchronize": [vp], "splash_ensemble_stream": [vp, C.POINTER(vp)],
        "splash_ensemble_get_state": [vp, C.c_int, dp],
        "splash_ensemble_member_info": [vp, C.c_int, dp, C.POINTER(C.c_uint32)],
        "splash_ensemble_schedule": [vp, ip, ip, dp],
        "splash_ensemble_size": [vp, ip, C.POINTER(C.c_int64)],
        "splash_ensemble_set_schedule": [vp, C.c_int, C.c_int],
        "splash_adjoint_create": [vp, C.c_int, C.POINTER(vp)],
        "splash_adjoint_destroy": [vp],
        "splash_adjoint_forward": [vp, dp, dp, C.c_int, C.c_double, dp],
        "splash_adjoint_backward": [vp, dp, dp, dp],
        "splash_adjoint_run": [vp, dp, dp, C.c_int, C.c_double, dp, dp, dp, dp],
        "splash_tlm_run": [vp, dp, dp, dp, dp, C.c_int, C.c_double, dp, dp],
        "splash_adjoint_branch_tape": [vp, dp, dp, C.c_int, C.c_int, dp, C.POINTER(C.c_int64)],
        "splash_adjoint_info": [vp, dp],
        "splash_adjoint_error_word": [vp, C.POINTER(C.c_uint32)],
        "splash_adjoint_dt_schedule": [vp, dp, C.c_int],
        "splash_face_geometry": [vp, dp, dp],
    }.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        msg = library().splash_last_error().decode(errors="replace")
        raise SplashError(f"splash error {rc}: {msg}")


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


# ---------------------------------------------------------------- meshes
@dataclass
class Mesh:
    """A mesh request: generated (kind, level) with the reference numbering,
    or explicit arrays (vertices [nv,3], face_offsets [nf+1], face_vertices)."""
    kind: int = MESH_ICOSPHERE_HEX
    level: int = 4
    vertices: np.ndarray | None = None
    face_offsets: np.ndarray | None = None
    face_vertices: np.ndarray | None = None
    _keep: list = field(default_factory=list, repr=False)

    def desc(self) -> MeshDesc:
        d = MeshDesc()
        d.kind = self.kind
        d.level = self.level
        if self.vertices is None:
            d.n_vertices = 0
            d.vertices = None
            d.n_faces = 0
            d.face_offsets = None
            d.face_vertices = None
        else:
            v = np.ascontiguousarray(self.vertices, dtype=np.float64).reshape(-1, 3)
            fo = np.ascontiguousarray(self.face_offsets, dtype=np.int32)
            fv = np.ascontiguousarray(self.face_vertices, dtype=np.int32)
            self._keep = [v, fo, fv]
            d.n_vertices = v.shape[0]
            d.vertices = _dptr(v)
            d.n_faces = fo.shape[0] - 1
            d.face_offsets = _iptr(fo)
            d.face_vertices = _iptr(fv)
        return d


def icosphere_hex(n: int) -> Mesh:
    """Dual of the n-times Loop-subdivided icosahedron (geometry/sph_gen.h:278)."""
    return Mesh(MESH_ICOSPHERE_HEX, n)


def quad_sphere(n: int) -> Mesh:
    """n-times Catmull-Clark-subdivided cube (geometry/sph_gen.h:286)."""
    return Mesh(MESH_QUAD_SPHERE, n)


def icosphere(n: int) -> Mesh:
    """n-times Loop-subdivided icosahedron (geometry/sph_gen.h:267)."""
    return Mesh(MESH_ICOSPHERE, n)


def n_faces_of(mesh: Mesh) -> int:
    if mesh.vertices is not None:
        return len(mesh.face_offsets) - 1
    if mesh.kind == MESH_ICOSPHERE_HEX:
        return 10 * 4 ** mesh.level + 2
    if mesh.kind == MESH_QUAD_SPHERE:
        return 6 * 4 ** mesh.level
    return 20 * 4 ** mesh.level


_GEOM_ARRAYS = {
    "vertices": (np.float64, 3), "face_off": (np.int32, 1), "face_vtx": (np.int32, 1),
    "nbr_off": (np.int32, 1), "nbr": (np.int32, 1), "nbr_edge": (np.int32, 1),
    "face_centers": (np.float64, 3), "normals": (np.float64, 3), "area": (np.float64, 1),
    "edge_normals": (np.float64, 3), "bm_dist": (np.float64, 1), "h_plus": (np.float64, 1),
    "h_minus": (np.float64, 1), "ff_plus": (np.int32, 2), "ff_minus": (np.int32, 2),
    "beta_plus": (np.float64, 2), "beta_minus": (np.float64, 2),
}


class Geometry:
    """Reference-numbered geometry (geometry/MUSCL_geometry.hpp:23-40) as numpy arrays."""

    def __init__(self, mesh: Mesh, threads: int = 0):
        lib = library()
        h = C.c_void_p()
        d = mesh.desc()
        _check(lib.splash_geometry_build(C.byref(d), threads, C.byref(h)))
        try:
            sizes = (C.c_int64 * 4)()
            scal = (C.c_double * 2)()
            _check(lib.splash_geometry_info(h, sizes, scal))
            self.n_vertices, self.n_faces, self.n_slots, self.max_slots = map(int, sizes)
            self.h0, self.round_diff = float(scal[0]), float(scal[1])
            self.arrays: dict[str, np.ndarray] = {}
            for name, (dt, width) in _GEOM_ARRAYS.items():
                nbytes = C.c_size_t()
                _check(lib.splash_geometry_get(h, name.encode(), None, 0, C.byref(nbytes)))
                a = np.empty(nbytes.value // np.dtype(dt).itemsize, dtype=dt)
                _check(lib.splash_geometry_get(h, name.encode(), a.ctypes.data_as(C.c_void_p),
                                               nbytes.value, None))
                self.arrays[name] = a.reshape(-1, width) if width > 1 else a
        finally:
            lib.splash_geometry_free(h)

    def __getitem__(self, name: str) -> np.ndarray:
        return self.arrays[name]

    def unit_face_centers(self) -> np.ndarray:
        fc = self.arrays["face_centers"]
        n = np.sqrt((fc[:, 0] * fc[:, 0] + fc[:, 1] * fc[:, 1]) + fc[:, 2] * fc[:, 2])
        return fc / n[:, None]


# ---------------------------------------------------------------- params
@dataclass
class SolverParams:
    """Keys read from input/parameters.json by the adiabatic constructor
    (physics/adiabatic.hpp:59-68); defaults are the reference's shipped file."""
    accretion_rate: float = 3.25e-7
    e_acc: float = 0.02
    omega_acc_abs: float = 0.4
    tilt_angle: float = 0.4
    acc_width: float = 0.1
    alpha: float = 1e-6
    friction_on: bool = True

    def to_c(self) -> Params:
        p = Params()
        p.accretion_rate = self.accretion_rate
        p.e_acc = self.e_acc
        p.omega_acc_abs = self.omega_acc_abs
        p.tilt_angle = self.tilt_angle
        p.acc_width = self.acc_width
        p.alpha = self.alpha
        p.friction_on = 1 if self.friction_on else 0
        return p

    def as_list(self) -> list[float]:
        return [self.accretion_rate, self.e_acc, self.omega_acc_abs, self.tilt_angle,
                self.acc_width, self.alpha, 1.0 if self.friction_on else 0.0]

    @classmethod
    def from_json(cls, path: str | os.PathLike) -> "SolverParams":
        with open(path) as f:
            d = json.load(f)
        return cls(accretion_rate=d["accretion_rate"], e_acc=d["e_acc"],
                   omega_acc_abs=d["omega_acc_abs"], tilt_angle=d["tilt_angle"],
                   acc_width=d["acc_width"], alpha=d["alpha"], friction_on=bool(d["friction_on"]))


# ---------------------------------------------------------------- solver
class Solver:
    """One GPU solver instance (C handle)."""

    def __init__(self, mesh: Mesh, U_in, dim: int, gam: float, omega_ns: float,
                 accretion_on: bool, params: SolverParams | None = None,
                 solver: int = SOLVER_HLLCPLUS, precision: int = PREC_FP64,
                 device: int = 0, threads: int = 0):
        lib = library()
        self._lib = lib
        self.handle = C.c_void_p()
        U = np.ascontiguousarray(U_in, dtype=np.float64)
        self.n_faces = U.shape[0] if U.ndim == 2 else U.size // dim
        self.dim = dim
        self.params = params or SolverParams()
        d = mesh.desc()
        p = self.params.to_c()
        _check(lib.splash_create(C.byref(d), _dptr(U), dim, gam, omega_ns,
                                 1 if accretion_on else 0, C.byref(p), solver, precision,
                                 device, threads, C.byref(self.handle)))

    def close(self) -> None:
        if self.handle:
            self._lib.splash_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # hot path
    def do_step(self, dt0: float) -> None:
        _check(self._lib.splash_do_step(self.handle, dt0))

    def do_steps(self, n: int, dt0: float) -> None:
        _check(self._lib.splash_do_steps(self.handle, n, dt0))

    def do_steps_host(self, U_in, n: int, dt0: float, out: np.ndarray | None = None) -> np.ndarray:
        """set_state(U_in), n steps and get_state() in one synchronising
        call (U_in None: continue from the current state)."""
        if out is None:
            out = np.empty((self.n_faces, self.dim))
        src = None if U_in is None else np.ascontiguousarray(U_in, dtype=np.float64)
        _check(self._lib.splash_do_steps_host(self.handle, None if src is None else _dptr(src), n, dt0,
                                              _dptr(out)))
        return out

    def synchronize(self) -> None:
        _check(self._lib.splash_synchronize(self.handle))

    def stream(self) -> int:
        """cudaStream_t of the solver, as an integer handle."""
        p = C.c_void_p()
        _check(self._lib.splash_stream(self.handle, C.byref(p)))
        return int(p.value or 0)

    def kernel_times(self, reps: int, dt0: float) -> np.ndarray:
        """Mean device ms per launch: dt, recon1, flux1, recon2, flux2."""
        out = np.zeros(5)
        _check(self._lib.splash_kernel_times(self.handle, reps, dt0, _dptr(out)))
        return out

    def launch_times(self, reps: int, dt0: float) -> np.ndarray:
        """Mean device ms of every timing slot of one step (mixed: the dt clip
        (an empty slot: the stage-1 edge launch clips dt), edge 1, update 1,
        edge 2, update 2; FP64: dt, recon1, flux1, recon2, flux2), with events
        between launches."""
        out = np.zeros(8)
        n = C.c_int(0)
        _check(self._lib.splash_launch_times(self.handle, reps, dt0, _dptr(out), 8, C.byref(n)))
        return out[: n.value].copy()

    def memory(self) -> tuple[int, int]:
        out = (C.c_int64 * 2)()
        _check(self._lib.splash_memory(self.handle, out))
        return int(out[0]), int(out[1])

    # accessors
    def time(self) -> float:
        t = C.c_double()
        _check(self._lib.splash_time(self.handle, C.byref(t)))
        return t.value

    def last_dt(self) -> float:
        t = C.c_double()
        _check(self._lib.splash_last_dt(self.handle, C.byref(t)))
        return t.value

    def get_stop_check(self) -> bool:
        s = C.c_int()
        _check(self._lib.splash_stop_check(self.handle, C.byref(s)))
        return bool(s.value)

    def error_word(self) -> int:
        b = C.c_uint32()
        _check(self._lib.splash_error_word(self.handle, C.byref(b)))
        return int(b.value)

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        U = out if out is not None else np.empty((self.n_faces, self.dim), dtype=np.float64)
        _check(self._lib.splash_get_state(self.handle, _dptr(U)))
        return U

    def set_state(self, U) -> None:
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(self._lib.splash_set_state(self.handle, _dptr(U)))

    def diagnostics(self) -> np.ndarray:
        out = np.zeros(5)
        _check(self._lib.splash_diagnostics(self.handle, _dptr(out)))
        return out

    def face_geometry(self) -> tuple[np.ndarray, np.ndarray]:
        """(unit face centres [F, 3], areas [F]) in reference face order."""
        c = np.empty((self.n_faces, 3))
        a = np.empty(self.n_faces)
        _check(self._lib.splash_face_geometry(self.handle, _dptr(c), _dptr(a)))
        return c, a

    def permutation(self) -> np.ndarray:
        p = np.empty(self.n_faces, dtype=np.int32)
        _check(self._lib.splash_get_permutation(self.handle, _iptr(p)))
        return p

    # writers (physics/adiabatic.hpp:101-348)
    def write_t_rho(self, path="results/rho.dat"):
        _check(self._lib.splash_write_t_rho(self.handle, str(path).encode()))

    def write_t_p(self, path="results/p.dat"):
        _check(self._lib.splash_write_t_p(self.handle, str(path).encode()))

    def write_t_curl(self, path="results/curl.dat"):
        _check(self._lib.splash_write_t_curl(self.handle, str(path).encode()))

    def write_t_omega_z(self, path="results/omega.dat"):
        _check(self._lib.splash_write_t_omega_z(self.handle, str(path).encode()))

    def write_t_L(self, px="results/Lx.dat", py="results/Ly.dat", pz="results/Lz.dat"):
        _check(self._lib.splash_write_t_L(self.handle, str(px).encode(), str(py).encode(),
                                          str(pz).encode()))

    def get_light_curves(self) -> list[float]:
        out = np.zeros(4)
        _check(self._lib.splash_get_light_curves(self.handle, _dptr(out)))
        return out.tolist()

    def write_final_state(self, path="results/final_state.dat"):
        _check(self._lib.splash_write_final_state(self.handle, str(path).encode()))


class _Named(Solver):
    _KIND = SOLVER_HLLCPLUS

    def __init__(self, mesh: Mesh, U_in, dim: int, gam: float, omega_ns: float = 0.0,
                 accretion_on: bool = False, threads: int = 0, *,
                 params: SolverParams | None = None, precision: int = PREC_FP64,
                 device: int = 0):
        super().__init__(mesh, U_in, dim, gam, omega_ns, accretion_on, params=params,
                         solver=self._KIND, precision=precision, device=device, threads=threads)


class MUSCL_HLLE(Solver):
    """Riemann_solvers/HLLE.hpp:11-13 (mesh, U_in, dim, gam, threads): the
    isothermal solver (dim 4; pressure a^2 Sigma with a = 1, no source)."""

    def __init__(self, mesh: Mesh, U_in, dim: int, gam: float, threads: int = 0, *,
                 precision: int = PREC_FP64, device: int = 0):
        super().__init__(mesh, U_in, dim, gam, 0.0, False, params=SolverParams(), solver=SOLVER_HLLE,
                         precision=precision, device=device, threads=threads)


class MUSCL_HLLE_p(_Named):
    """Riemann_solvers/HLLE_p.hpp:11-13 (mesh, U_in, dim, gam, omega_ns, accretion_on, threads)."""
    _KIND = SOLVER_HLLE_P


class MUSCL_HLLC(_Named):
    """Riemann_solvers/HLLC.hpp:11-13 (mesh, U_in, dim, gam, omega_ns, accretion_on, threads)."""
    _KIND = SOLVER_HLLC


class MUSCL_HLLCplus(_Named):
    """Riemann_solvers/HLLCplus.hpp:11-13 (mesh, U_in, dim, gam, omega_ns, accretion_on, threads)."""
    _KIND = SOLVER_HLLCPLUS


class Ensemble:
    """Many independent solvers advanced together (FP32/FP64 mixed).

    members: list of dicts with keys mesh (Mesh), U_in, gam, omega_ns,
    accretion_on, params (SolverParams), solver."""

    def __init__(self, members, device: int = 0, autotune: bool = True):
        lib = library()
        self._lib = lib
        self.handle = C.c_void_p()
        self._keep = []
        arr = (Member * len(members))()
        self.n_faces = []
        self.dims = []
        for i, m in enumerate(members):
            U = np.ascontiguousarray(m["U_in"], dtype=np.float64)
            self._keep.append(U)
            mesh = m["mesh"]
            arr[i].mesh_kind = mesh.kind
            arr[i].level = mesh.level
            arr[i].U_in = _dptr(U)
            arr[i].gam = m["gam"]
            arr[i].omega_ns = m.get("omega_ns", 0.0)
            arr[i].accretion_on = 1 if m.get("accretion_on", False) else 0
            arr[i].params = (m.get("params") or SolverParams()).to_c()
            arr[i].solver_kind = m.get("solver", SOLVER_HLLCPLUS)
            self.n_faces.append(U.shape[0])
            self.dims.append(4 if arr[i].solver_kind == SOLVER_HLLE else 5)
        _check(lib.splash_ensemble_create(arr, len(members), device, 1 if autotune else 0,
                                          C.byref(self.handle)))
        self._keep = []

    def close(self):
        if self.handle:
            self._lib.splash_ensemble_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def do_steps(self, n: int, dt0: float) -> None:
        _check(self._lib.splash_ensemble_do_steps(self.handle, n, dt0))

    def synchronize(self) -> None:
        _check(self._lib.splash_ensemble_synchronize(self.handle))

    def stream(self) -> int:
        p = C.c_void_p()
        _check(self._lib.splash_ensemble_stream(self.handle, C.byref(p)))
        return int(p.value or 0)

    def get_state(self, member: int) -> np.ndarray:
        U = np.empty((self.n_faces[member], self.dims[member]))
        _check(self._lib.splash_ensemble_get_state(self.handle, member, _dptr(U)))
        return U

    def member_info(self, member: int) -> dict:
        out = np.zeros(4)
        err = C.c_uint32()
        _check(self._lib.splash_ensemble_member_info(self.handle, member, _dptr(out), C.byref(err)))
        return {"t": out[0], "dt": out[1], "max_vel": out[2], "extra_dt": out[3], "err": int(err.value)}

    def schedule(self) -> dict:
        """The schedule in use: tile order, edge block width (0: the
        persistent launch), and the autotuner's ms per step of every
        candidate (five-launch rows by order x {32, 64, 128} threads, and
        the persistent launch by order)."""
        o = C.c_int()
        w = C.c_int()
        ms = np.zeros(12)
        _check(self._lib.splash_ensemble_schedule(self.handle, C.byref(o), C.byref(w), _dptr(ms)))
        return {"order": ["member", "largest-first", "round-robin"][o.value], "recon_width": w.value,
                "persistent": w.value == 0, "trial_ms": ms[:9].reshape(3, 3).tolist(),
                "trial_ms_persistent": ms[9:].tolist()}

    def set_schedule(self, order: int, edge_block: int) -> None:
        """order 0..2 (member, largest first, round-robin); edge_block 32,
        64 or 128 threads (five launches per step) or 0 (one persistent
        launch per do_steps call)."""
        _check(self._lib.splash_ensemble_set_schedule(self.handle, order, edge_block))

    def size(self) -> tuple[int, int]:
        n = C.c_int()
        t = C.c_int64()
        _check(self._lib.splash_ensemble_size(self.handle, C.byref(n), C.byref(t)))
        return n.value, t.value


class Adjoint:
    """Tangent-linear model and discrete adjoint of n FP64 do_step calls.

    ``base`` is an FP64 :class:`Solver` whose mesh, solver kind, gam,
    omega_ns and parameters define the map; theta = (accretion_rate,
    tilt_angle, omega_acc_abs).  The dt schedule of the forward run is
    frozen (the derivative of the CFL min() on the branch taken).  States
    are [n_faces, 5] arrays in reference face order."""

    def __init__(self, base: Solver, checkpoint_every: int = 50):
        lib = library()
        self._lib = lib
        self.base = base  # the adjoint borrows its geometry
        self.n_faces = base.n_faces
        self.handle = C.c_void_p()
        _check(lib.splash_adjoint_create(base.handle, checkpoint_every, C.byref(self.handle)))

    def close(self):
        if self.handle:
            self._lib.splash_adjoint_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _arr(a, shape=None):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        if shape is not None and a.size != int(np.prod(shape)):
            raise ValueError(f"expected {shape} values, got {a.shape}")
        return a

    def _p(self, a):
        return _dptr(a) if a is not None else None

    def forward(self, U0, theta, n_steps: int, dt0: float) -> np.ndarray:
        U0 = self._arr(U0, (self.n_faces, 5))
        th = self._arr(theta, (3,))
        out = np.empty((self.n_faces, 5))
        _check(self._lib.splash_adjoint_forward(self.handle, _dptr(U0), self._p(th), n_steps, dt0, _dptr(out)))
        return out

    def backward(self, lambda_final) -> tuple[np.ndarray, np.ndarray]:
        lam = self._arr(lambda_final, (self.n_faces, 5))
        gU = np.empty((self.n_faces, 5))
        gth = np.empty(3)
        _check(self._lib.splash_adjoint_backward(self.handle, _dptr(lam), _dptr(gU), _dptr(gth)))
        return gU, gth

    def run(self, U0, theta, n_steps: int, dt0: float, sigma_target) -> tuple[float, np.ndarray, np.ndarray]:
        """loss = 1/2 sum area (Sigma_final - sigma_target)^2 and its gradients."""
        U0 = self._arr(U0, (self.n_faces, 5))
        th = self._arr(theta, (3,))
        tgt = self._arr(sigma_target, (self.n_faces,))
        loss = C.c_double()
        gU = np.empty((self.n_faces, 5))
        gth = np.empty(3)
        _check(self._lib.splash_adjoint_run(self.handle, _dptr(U0), self._p(th), n_steps, dt0, _dptr(tgt),
                                            C.byref(loss), _dptr(gU), _dptr(gth)))
        return loss.value, gU, gth

    def tlm(self, U0, theta, dU0, dtheta, n_steps: int, dt0: float) -> tuple[np.ndarray, np.ndarray]:
        U0 = self._arr(U0, (self.n_faces, 5))
        th = self._arr(theta, (3,))
        dU = self._arr(dU0, (self.n_faces, 5))
        dth = self._arr(dtheta, (3,))
        U = np.empty((self.n_faces, 5))
        dUf = np.empty((self.n_faces, 5))
        _check(self._lib.splash_tlm_run(self.handle, _dptr(U0), self._p(th), self._p(dU), self._p(dth), n_steps,
                                        dt0, _dptr(U), _dptr(dUf)))
        return U, dUf

    _TAPE_MODES = {"replay": 0, "record": 1, "compare": 2}

    def branch_tape(self, U0, theta, n_steps: int, mode: str) -> tuple[np.ndarray, int]:
        """The FP64 forward on the last forward run's dt schedule with its
        branch decisions taped (validation only): mode "record" records them,
        "replay" replays the recording (the branch-frozen map the adjoint
        differentiates; count = replayed decisions the run's own values would
        have taken otherwise), "compare" runs the plain forward and counts
        the (face, launch) evaluations whose branch path departs from the
        recording.  Returns (U_final, count)."""
        U0 = self._arr(U0, (self.n_faces, 5))
        th = self._arr(theta, (3,))
        out = np.empty((self.n_faces, 5))
        count = C.c_int64(0)
        _check(self._lib.splash_adjoint_branch_tape(self.handle, _dptr(U0), self._p(th), n_steps,
                                                    self._TAPE_MODES[mode], _dptr(out), C.byref(count)))
        return out, count.value

    def info(self) -> dict:
        o = np.zeros(8)
        _check(self._lib.splash_adjoint_info(self.handle, _dptr(o)))
        return {"steps": int(o[0]), "clipped_steps": int(o[1]), "dt_min": o[2], "dt_max": o[3],
                "ms_forward": o[4], "ms_backward": o[5], "ms_tlm": o[6], "device_bytes": int(o[7])}

    def error_word(self) -> int:
        e = C.c_uint32()
        _check(self._lib.splash_adjoint_error_word(self.handle, C.byref(e)))
        return int(e.value)

    def dt_schedule(self) -> np.ndarray:
        n = self.info()["steps"]
        d = np.empty(max(n, 1))
        _check(self._lib.splash_adjoint_dt_schedule(self.handle, _dptr(d), len(d)))
        return d[:n]


def read_input_dat(path, n_faces: int, dim: int) -> np.ndarray:
    """input/input.dat reader with the rule of test.cpp:48-77 (missing values = 1)."""
    vals = np.array(Path(path).read_text().split(), dtype=np.float64)
    need = n_faces * dim
    if vals.size < need:
        vals = np.concatenate([vals, np.ones(need - vals.size)])
    return vals[:need].reshape(n_faces, dim)


def read_final_state(path, n_faces: int, dim: int) -> np.ndarray:
    """results/final_state.dat as a restart state: the reference restarts by
    reading that file in place of input/input.dat (test.cpp:34-35), with the
    same reader rule; the file holds six significant digits per value
    (physics/adiabatic.hpp:335-348), so a restart starts from the rounded
    state, as the reference's does."""
    return read_input_dat(path, n_faces, dim)


def format_final_state(U) -> str:
    """The text write_final_state produces for a state U [F, dim] in
    reference face order: every value in the C++ stream's default format
    (%g, six significant digits) followed by a space, one row per face
    (physics/adiabatic.hpp:335-348)."""
    return "".join("".join(f"{x:g} " for x in row) + "\n" for row in np.asarray(U, dtype=np.float64))
