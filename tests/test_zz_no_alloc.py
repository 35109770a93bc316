"""splash_cfl_dt_noalloc: the allocation-free CFL clip for callers that
cannot allocate device memory when they need the time step (a coupling code
whose device memory is all owned by its own pool, or code about to capture
its stream into a CUDA graph).

The test owns every device buffer (allocated here through torch, not by the
library), calls the entry point through the C ABI twice in a row on two
successive states, and checks each result against what the solver's own
path (splash_do_step -> splash_last_dt, splash_diagnostics) reports for the
same state, at the FP64 tolerance of the other tests (1e-10 relative).
This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from helpers import mesh_of

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _noalloc(lib, torch, U, r, area, h0, gam, dt0):
    dU = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    dr = torch.from_numpy(np.ascontiguousarray(r)).cuda()
    da = torch.from_numpy(np.ascontiguousarray(area)).cuda()
    out = torch.full((9,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.splash_cfl_dt_noalloc(C.c_void_p(dU.data_ptr()), C.c_void_p(dr.data_ptr()),
                                   C.c_void_p(da.data_ptr()), U.shape[0], gam, 0.0, 1e-6, h0, dt0,
                                   C.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.splash_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_cfl_matches_solver_two_calls():
    torch = pytest.importorskip("torch")
    import splash_gb300 as sg

    lib = sg.library()
    lib.splash_cfl_dt_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_void_p, C.c_void_p]
    lib.splash_cfl_dt_noalloc.restype = C.c_int
    mesh = mesh_of("hex", 5)
    g = sg.Geometry(mesh)
    r = g.unit_face_centers()
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(r, gam, seed=9)
    dt0 = 1.0  # large, so the CFL clip decides dt
    s = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, True,
                          params=sg.SolverParams(accretion_rate=1e-2, e_acc=0.5, omega_acc_abs=0.5,
                                                 tilt_angle=0.2, acc_width=0.1))
    diag0 = s.diagnostics()
    s.do_step(dt0)
    dt_a = s.last_dt()
    U1 = s.get_state()
    diag1 = s.diagnostics()
    s.do_step(dt0)
    dt_b = s.last_dt()
    s.close()

    out_a = _noalloc(lib, torch, U0, r, g["area"], g.h0, gam, dt0)
    out_b = _noalloc(lib, torch, U1, r, g["area"], g.h0, gam, dt0)
    assert dt_a < dt0 and dt_b < dt0  # the clip is active
    # dt is a min/max of the same FP64 candidates: exact in any order
    assert out_a[0] == dt_a, (out_a[0], dt_a)
    assert out_b[0] == dt_b, (out_b[0], dt_b)
    # the sums are reduced in another order: equal to rounding
    assert np.allclose(out_a[4:], diag0, rtol=TOL, atol=0), (out_a[4:], diag0)
    assert np.allclose(out_b[4:], diag1, rtol=TOL, atol=0), (out_b[4:], diag1)
    assert out_a[3] == 0.0 and out_b[3] == 0.0
    # the clip formula itself: dt = 0.1 h0 / max_vel
    assert abs(out_a[0] - 0.1 * g.h0 / out_a[1]) <= 1e-15 * out_a[0]


def test_noalloc_rejects_oversized_input():
    import splash_gb300 as sg

    lib = sg.library()
    lib.splash_cfl_dt_noalloc.restype = C.c_int
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.splash_cfl_dt_noalloc(dummy, dummy, dummy, C.c_int(4194305), C.c_double(1.25),
                                   C.c_double(0.0), C.c_double(1e-6), C.c_double(0.01),
                                   C.c_double(1e-3), dummy, None)
    assert rc == 1
    assert b"4194304" in lib.splash_last_error()
