"""GPU parity: the CUDA FP64 path through the C ABI against the reference's
own output (committed golden states) and against the CPU oracle.

Tolerance: 1e-10 relative L-infinity per conserved field (max |GPU - ref| /
max |ref| over faces), the bar for the FP64 plain method; dt, t and the
stop flag must agree as well."""
import numpy as np
import pytest

from helpers import load, make_oracle, mesh_of, rel_linf

pytestmark = pytest.mark.gpu

TOL = 1e-10
STATE_CASES = ["c0_hex4_hllep", "c1_hex4_hllcp", "hex3_hllc_acc", "hex3_hllcp_acc",
               "hex3_hllcp_nofric", "quad3_hllc_acc", "shear_quad4_hllc"]


def gpu_solver(case, precision=0):
    import splash_gb300 as sg

    p = case["params"]
    params = sg.SolverParams(accretion_rate=p[0], e_acc=p[1], omega_acc_abs=p[2], tilt_angle=p[3],
                             acc_width=p[4], alpha=p[5], friction_on=bool(p[6]))
    return sg.Solver(mesh_of(str(case["mesh"]), int(case["level"])), case["U0"], 5,
                     float(case["gam"]), 0.0, bool(case["accretion_on"]), params=params,
                     solver=int(case["solver"]), precision=precision, device=0)


@pytest.mark.parametrize("case_name", STATE_CASES)
def test_fp64_matches_reference_states(case_name):
    c = load(f"state_{case_name}.npz")
    s = gpu_solver(c)
    done = 0
    for k, nstep in enumerate(c["steps"]):
        s.do_steps(int(nstep) - done, float(c["dt0"]))
        done = int(nstep)
        U = s.get_state()
        err = rel_linf(U, c["U"][k])
        assert np.all(err < TOL), (case_name, int(nstep), err)
        assert abs(s.last_dt() - c["dt"][k]) <= 1e-13 * c["dt"][k], (s.last_dt(), c["dt"][k])
        assert abs(s.time() - c["t"][k]) <= 1e-12 * c["t"][k]
        assert s.get_stop_check() == bool(c["stop"][k])
    s.close()


@pytest.mark.parametrize("kind,level,solver,acc", [("hex", 5, 3, True), ("hex", 6, 2, True),
                                                   ("quad", 5, 1, False)])
def test_fp64_matches_oracle_larger_mesh(kind, level, solver, acc):
    """Larger meshes than the committed fixtures: GPU vs the CPU oracle
    (itself bit-identical to the reference), 40 steps."""
    import splash_gb300 as sg

    g = sg.Geometry(mesh_of(kind, level))
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=level)
    case = {"U0": U0, "gam": gam, "accretion_on": acc, "solver": solver, "mesh": kind,
            "level": level, "params": np.array([1e-2, 0.5, 0.5, 0.2, 0.1, 1e-6, 1.0])}
    o = make_oracle(g, case)
    s = gpu_solver(case)
    for chunk in (1, 9, 30):
        o.do_steps(chunk, 1e-3)
        s.do_steps(chunk, 1e-3)
        err = rel_linf(s.get_state(), o.get_state())
        assert np.all(err < TOL), (kind, level, solver, err)
    info = o.info()
    assert abs(s.time() - info["t"]) <= 1e-12 * info["t"]
    s.close()


def test_fp64_mid_size_workload_100_steps():
    """The accreting mid-size workload itself: icosphere_hex(7) (163,842
    faces), MUSCL_HLLCplus, accretion on (rate 1e-2, e_acc 0.5, omega_acc
    0.5, tilt 0.2, width 0.1, friction on), quiet noise of seed 1, dt0 =
    2e-4, 100 steps.  The GPU FP64 state is compared with the oracle on every
    face and with the reference's own state (state_c1_hex7_hllcp.npz, written
    by the reference on every 61st face) at 1e-10 relative L-infinity per
    field; dt, t and the stop flag equal."""
    import hashlib

    import splash_gb300 as sg

    c = load("state_c1_hex7_hllcp.npz")
    g = sg.Geometry(mesh_of(str(c["mesh"]), int(c["level"])))
    U0 = sg.initial_conditions.quiet_noise(g.unit_face_centers(), float(c["gam"]), seed=int(c["seed"]))
    assert hashlib.sha256(np.ascontiguousarray(U0, "<f8").tobytes()).hexdigest() == str(c["U0_sha256"])
    case = {k: c[k] for k in ("gam", "accretion_on", "solver", "mesh", "level", "params")}
    case["U0"] = U0
    nsteps, dt0 = int(c["steps"]), float(c["dt0"])
    s = gpu_solver(case)
    s.do_steps(nsteps, dt0)
    U = s.get_state()
    # the reference's own faces
    idx = c["index"]
    err_ref = np.max(np.abs(U[idx] - c["U_subset"]), axis=0) / c["U_absmax"]
    assert np.all(err_ref < TOL), err_ref
    assert abs(s.last_dt() - float(c["dt"])) <= 1e-13 * float(c["dt"])
    assert abs(s.time() - float(c["t"])) <= 1e-12 * float(c["t"])
    assert s.get_stop_check() == bool(c["stop"])
    # every face against the oracle
    o = make_oracle(g, case)
    o.do_steps(nsteps, dt0)
    err = rel_linf(U, o.get_state())
    assert np.all(err < TOL), err
    s.close()


@pytest.mark.parametrize("solver", [1, 2])
def test_fp64_mid_size_workload_other_solvers(solver):
    """The same hex(7) accreting workload (quiet noise of seed 1, dt0 = 2e-4,
    100 steps) with MUSCL_HLLE_p and MUSCL_HLLC: the GPU FP64 state against
    the oracle on every face at 1e-10 relative L-infinity per field, dt, t
    and the stop flag equal."""
    import splash_gb300 as sg

    c = load("state_c1_hex7_hllcp.npz")
    g = sg.Geometry(mesh_of(str(c["mesh"]), int(c["level"])))
    U0 = sg.initial_conditions.quiet_noise(g.unit_face_centers(), float(c["gam"]), seed=int(c["seed"]))
    case = {k: c[k] for k in ("gam", "accretion_on", "mesh", "level", "params")}
    case["U0"] = U0
    case["solver"] = solver
    nsteps, dt0 = int(c["steps"]), float(c["dt0"])
    s = gpu_solver(case)
    s.do_steps(nsteps, dt0)
    o = make_oracle(g, case)
    o.do_steps(nsteps, dt0)
    err = rel_linf(s.get_state(), o.get_state())
    assert np.all(err < TOL), (solver, err)
    info = o.info()
    assert abs(s.last_dt() - info["dt"]) <= 1e-13 * info["dt"]
    assert abs(s.time() - info["t"]) <= 1e-12 * info["t"]
    assert s.get_stop_check() == info["stop"]
    s.close()


def test_step_is_deterministic_and_graph_replay_equals_single_steps():
    c = load("state_hex3_hllcp_acc.npz")
    a = gpu_solver(c)
    b = gpu_solver(c)
    a.do_steps(20, float(c["dt0"]))
    for _ in range(20):
        b.do_step(float(c["dt0"]))
    assert np.array_equal(a.get_state(), b.get_state())


def test_state_round_trip_and_permutation():
    c = load("state_hex3_hllc_acc.npz")
    s = gpu_solver(c)
    assert np.array_equal(s.get_state(), c["U0"])
    p = s.permutation()
    assert np.array_equal(np.sort(p), np.arange(len(p)))
    U = c["U0"].copy()
    U[:, 0] *= 1.01
    s.set_state(U)
    assert np.array_equal(s.get_state(), U)


def test_stop_flag_bits_negative_extra_dt():
    """u_phi = 0.5 > sqrt(GM) makes g_eff < 0, so extra_dt_constr is negative
    and the reference latches stop_check (physics/adiabatic.hpp:566-577)."""
    import splash_gb300 as sg

    c = load("state_shear_quad4_hllc.npz")
    s = gpu_solver(c)
    assert not s.get_stop_check()
    s.do_step(float(c["dt0"]))
    assert s.error_word() & sg.STOP_NEG_EXTRA_DT


@pytest.mark.parametrize("field", [0, 4])
def test_nan_input_stop_flag_matches_reference(field):
    """A NaN planted in the host input state (never on the device).  In the
    density it reaches the fluxes and latches the stop flag
    (MUSCL_base.hpp:264-268, adiabatic.hpp:671-676); in the energy the
    pressure floor swallows it (MUSCL_base.hpp:538) and the reference does not
    stop.  The GPU error word must equal the oracle's stop bits."""
    import splash_gb300 as sg

    c = load("state_hex3_hllc_acc.npz")
    U = c["U0"].copy()
    U[5, field] = np.nan
    c2 = dict(c)
    c2["U0"] = U
    o = make_oracle(sg.Geometry(mesh_of("hex", 3)), c2)
    bits = o.do_step(1e-3)
    s = gpu_solver(c)
    s.set_state(U)
    s.do_step(1e-3)
    assert s.error_word() == bits
    assert s.get_stop_check() == (field == 0)
    assert np.array_equal(np.isnan(s.get_state()), np.isnan(o.get_state()))


@pytest.mark.parametrize("precision", [0, 1])
def test_state_transfer_paths_agree(monkeypatch, precision):
    """States cross the C ABI either directly (the device reads and writes the
    caller's host array over a coherent link, when the device reports
    pageable-memory access) or through a pinned staging buffer
    (SPLASH_STAGED_TRANSFERS set): both round-trip bit for bit and give the
    same run."""
    import splash_gb300 as sg

    mesh = mesh_of("hex", 4)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=11)
    monkeypatch.delenv("SPLASH_STAGED_TRANSFERS", raising=False)
    a = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, False, precision=precision)
    monkeypatch.setenv("SPLASH_STAGED_TRANSFERS", "1")
    b = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, False, precision=precision)
    for s in (a, b):
        assert np.array_equal(s.get_state(), U0)
        s.set_state(U0[::-1].copy())
        assert np.array_equal(s.get_state(), U0[::-1])
        s.set_state(U0)
        s.do_steps(3, 1e-3)
    assert np.array_equal(a.get_state(), b.get_state())


@pytest.mark.parametrize("precision", [0, 1])
def test_device_diagnostics_and_light_curves(precision):
    """Mass / angular momentum / energy sums and the four light curves
    (physics/adiabatic.hpp:228-333) reduced on the device, against the same
    sums over the downloaded state on the host (summation order differs)."""
    import splash_gb300 as sg

    mesh = mesh_of("hex", 4)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    r = g.unit_face_centers()
    U0 = sg.initial_conditions.rotating_blob(r, gam, seed=12)
    s = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, False, precision=precision)
    s.do_steps(5, 1e-3)
    U = s.get_state()
    area = g["area"]
    d = s.diagnostics()
    assert np.allclose(d, (U * area[:, None]).sum(axis=0), rtol=1e-12, atol=1e-15)
    # light curves on the host with the reference's expressions
    fc = g["face_centers"]
    nrm = np.sqrt((fc[:, 0] * fc[:, 0] + fc[:, 1] * fc[:, 1]) + fc[:, 2] * fc[:, 2])
    fcn = fc / nrm[:, None]
    vel = np.cross(fcn, U[:, 1:4]) / (-U[:, 0])[:, None]
    n = np.sqrt(np.sum(vel * vel, axis=1))
    PI = np.maximum(1e-16, (U[:, 4] - U[:, 0] * (n * n) / 2) * (gam - 1))
    D = 9.4 * 3 * 1e19 / 15000
    obs = [np.array([D, 0, 0]), np.array([np.sqrt(D), 0, np.sqrt(D)]), np.array([0, 0, D]), np.array([0, 0, -D])]
    phi = np.arctan2(fc[:, 1] / nrm, fc[:, 0] / nrm)
    theta = np.arccos(fc[:, 2] / nrm)
    seen = [(phi < np.pi / 2) & (phi > -np.pi / 2), fcn @ obs[1] > 0, theta < np.pi / 2, theta > np.pi / 2]
    ref = [np.sum((PI * (np.abs(fcn @ o) / np.linalg.norm(o)) * area)[m]) for o, m in zip(obs, seen)]
    assert np.allclose(s.get_light_curves(), ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("precision", [0, 1])
def test_do_steps_host_equals_separate_calls(precision):
    """splash_do_steps_host (upload, n steps, download, one synchronisation)
    gives exactly the states of set_state + do_steps + get_state, with the
    input and output arrays distinct or the same; NULL input continues."""
    import splash_gb300 as sg

    mesh = mesh_of("hex", 4)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=21)
    a = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, True, precision=precision)
    b = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, True, precision=precision)
    U1 = U0.copy()
    U1[:, 0] *= 1.001
    a.set_state(U1)
    a.do_steps(3, 1e-3)
    ref = a.get_state()
    out = b.do_steps_host(U1, 3, 1e-3)
    assert np.array_equal(out, ref)
    a.do_steps(2, 1e-3)
    assert np.array_equal(b.do_steps_host(None, 2, 1e-3), a.get_state())
    inout = U1.copy()
    b.do_steps_host(inout, 3, 1e-3, out=inout)
    assert np.array_equal(inout, ref)
