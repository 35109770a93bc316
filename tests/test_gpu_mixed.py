"""FP32/FP64 mixed path: accuracy against the FP64 path (itself at 1e-10
of the reference), conservation, and behaviour parity (stop flags, API)."""
import numpy as np
import pytest

from helpers import load, mesh_of, rel_linf

pytestmark = pytest.mark.gpu


def make(case, precision):
    from test_gpu_parity import gpu_solver

    return gpu_solver(case, precision=precision)


def l1_rel(a, b, area):
    """Area-weighted relative L1 per field: sum A|a-b| / sum A|b|."""
    num = np.sum(area[:, None] * np.abs(a - b), axis=0)
    den = np.sum(area[:, None] * np.abs(b), axis=0)
    return num / np.where(den > 0, den, 1)


def test_accreting_mid_size_2000_steps():
    """icosphere_hex(7), HLLC+, accretion on, Sigma = Pi = 1 +- 1e-3, 2000
    steps at dt0 = 2e-4: relative L1 density error of the mixed path below
    1e-5 against FP64 (the stated accuracy bar)."""
    import splash_gb300 as sg

    g = sg.Geometry(mesh_of("hex", 7))
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.quiet_noise(g.unit_face_centers(), gam, seed=1)
    case = {"U0": U0, "gam": gam, "accretion_on": True, "solver": 3, "mesh": "hex", "level": 7,
            "params": np.array([1e-2, 0.5, 0.5, 0.2, 0.1, 1e-6, 1.0])}
    a = make(case, 0)
    b = make(case, 1)
    a.do_steps(2000, 2e-4)
    b.do_steps(2000, 2e-4)
    Ua, Ub = a.get_state(), b.get_state()
    err = l1_rel(Ub, Ua, g["area"])
    assert err[0] < 1e-5, err
    assert np.all(np.isfinite(Ub))
    assert abs(a.time() - b.time()) < 1e-9 * a.time()
    # mass budget: both paths gain the same mass from accretion
    ma, mb = np.sum(g["area"] * Ua[:, 0]), np.sum(g["area"] * Ub[:, 0])
    assert abs(ma - mb) < 1e-9 * ma


@pytest.mark.parametrize("case_name,tol", [("c0_hex4_hllep", 2e-5), ("hex3_hllc_acc", 2e-5),
                                           ("hex3_hllcp_acc", 2e-5), ("hex3_hllcp_nofric", 2e-5),
                                           ("quad3_hllc_acc", 2e-5), ("c1_hex4_hllcp", 1e-6)])
def test_mixed_close_to_reference_states(case_name, tol):
    """Against the reference's own states: relative L-infinity per field."""
    c = load(f"state_{case_name}.npz")
    s = make(c, 1)
    done = 0
    for k, nstep in enumerate(c["steps"]):
        s.do_steps(int(nstep) - done, float(c["dt0"]))
        done = int(nstep)
    U, R = s.get_state(), c["U"][-1]
    err = rel_linf(U, R)
    # density and energy: relative to their own magnitude
    assert err[0] < tol and err[4] < tol, (case_name, err)
    # angular momentum starts at ~0 in the accreting case, so it is measured
    # against the momentum scale Sigma * c_s rather than against max |l|
    gam = float(c["gam"])
    scale = np.max(R[:, 0] * np.sqrt(gam * (gam - 1) * R[:, 4] / R[:, 0]))
    assert np.max(np.abs(U[:, 1:4] - R[:, 1:4])) < tol * scale, (case_name, err)
    assert s.get_stop_check() == bool(c["stop"][-1])


def test_mixed_stop_flags_and_round_trip():
    import splash_gb300 as sg

    c = load("state_shear_quad4_hllc.npz")
    s = make(c, 1)
    assert np.array_equal(s.get_state(), c["U0"])
    s.do_step(float(c["dt0"]))
    assert s.error_word() & sg.STOP_NEG_EXTRA_DT
    U = c["U0"].copy()
    U[3, 0] = np.nan
    s.set_state(U)
    s.do_step(1e-3)
    assert s.error_word() & sg.STOP_NAN_FLUX


def test_mass_conservation_without_sources():
    """Accretion off: the total mass changes only through the flux
    asymmetry; FP64 keeps it to round-off and the mixed path to FP32 flux
    precision."""
    import splash_gb300 as sg

    g = sg.Geometry(mesh_of("hex", 6))
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=3)
    case = {"U0": U0, "gam": gam, "accretion_on": False, "solver": 2, "mesh": "hex", "level": 6,
            "params": np.array([1e-2, 0.5, 0.5, 0.2, 0.1, 1e-6, 1.0])}
    m0 = np.sum(g["area"] * U0[:, 0])
    for prec, tol in ((0, 1e-12), (1, 1e-7)):
        s = make(case, prec)
        s.do_steps(200, 1e-3)
        m = np.sum(g["area"] * s.get_state()[:, 0])
        assert abs(m / m0 - 1) < tol, (prec, m / m0 - 1)


def test_cold_rotating_flow():
    """Kinetic energy 84 times the thermal energy (solid-body rotation at
    Mach ~25, Pi = 1e-4 Sigma^gam): the pressure recovered from the FP64
    state, E - |r x l|^2 / (2 Sigma), cancels two digits, which the
    double-word recovery of the face state absorbs.  400 steps on hex(6),
    HLLC+, accretion off: measured relative L1 against FP64 1.0e-7 (Sigma),
    1.9e-7 (E), 3.0e-6 (Pi), the same as with an FP64 recovery to three
    digits."""
    import splash_gb300 as sg

    mesh = sg.icosphere_hex(6)
    g = sg.Geometry(mesh)
    r = g.unit_face_centers()
    area = g["area"]
    gam = sg.initial_conditions.gam2d(4 / 3)
    rng = np.random.default_rng(5)
    c = rng.normal(size=3)
    c /= np.linalg.norm(c)
    sigma = 1 + 0.2 * np.exp(-np.sum((r - c) ** 2, axis=1) / 0.05)
    pi = 1e-4 * sigma ** gam
    v = 0.3 * np.cross(np.array([0.0, 0.0, 1.0]), r)
    U0 = sg.initial_conditions.to_conserved(r, sigma, pi, v, gam)
    out = {}
    for prec in (sg.PREC_MIXED, sg.PREC_FP64):
        s = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, False, precision=prec)
        s.do_steps(400, 1e-3)
        assert not s.get_stop_check()
        out[prec] = s.get_state()
        s.close()
    Um, U6 = out[sg.PREC_MIXED], out[sg.PREC_FP64]

    def l1(a, b):
        return np.sum(area * np.abs(a - b)) / np.sum(area * np.abs(b))

    def pressure(U):
        cr = np.cross(r, U[:, 1:4])
        return (U[:, 4] - 0.5 * np.sum(cr * cr, axis=1) / U[:, 0]) * (gam - 1)

    assert l1(Um[:, 0], U6[:, 0]) < 1e-6
    assert l1(Um[:, 4], U6[:, 4]) < 1e-6
    assert l1(pressure(Um), pressure(U6)) < 1e-5


def test_mixed_dt0_changes_between_steps():
    """do_step(dt0) with a different dt0 on every call: the captured step's
    dt0 argument is rewritten in the instantiated graph and each step uses
    its own dt0 (unclipped here), like MUSCL_base.hpp:100."""
    c = load("state_hex3_hllcp_acc.npz")
    s = make(c, 1)
    t = 0.0
    for dt0 in (1e-3, 5e-4, 5e-4, 2e-4, 1e-3):
        s.do_step(dt0)
        assert s.last_dt() == dt0
        t += dt0
    assert abs(s.time() - t) < 1e-15
    # the same sequence on the FP64 path gives the same times
    f = make(c, 0)
    for dt0 in (1e-3, 5e-4, 5e-4, 2e-4, 1e-3):
        f.do_step(dt0)
    assert abs(f.time() - s.time()) < 1e-15


@pytest.mark.parametrize("solver", [2, 4])
def test_mixed_edge_state_writer_matches_fp64(tmp_path, solver):
    """write_t_curl reads the last stage's edge states; the mixed path keeps
    them edge-major (two sides per edge) and the writer maps every slot to
    its edge and side.  After the same steps the mixed and FP64 writers must
    agree to mixed-precision tolerance (a wrong slot mapping scrambles the
    per-face vorticity by O(1))."""
    import splash_gb300 as sg

    mesh = mesh_of("hex", 4)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=4)
    dim = 4 if solver == 4 else 5
    U0 = np.ascontiguousarray(U0[:, :dim])
    out = {}
    for prec in (sg.PREC_FP64, sg.PREC_MIXED):
        s = sg.Solver(mesh, U0, dim, gam, 0.0, False, params=sg.SolverParams(), solver=solver, precision=prec)
        s.do_steps(20, 1e-3)
        path = tmp_path / f"curl_{prec}.dat"
        s.write_t_curl(path)
        out[prec] = np.array(path.read_text().split(), dtype=float)
        s.close()
    a, b = out[sg.PREC_FP64], out[sg.PREC_MIXED]
    assert a.shape == b.shape == (g.n_faces + 1,)
    scale = np.max(np.abs(a[1:]))
    assert scale > 0
    assert np.max(np.abs(a[1:] - b[1:])) < 1e-4 * scale


def test_multi_step_graphs_equal_single_steps():
    """do_steps(n) replays graphs of several steps (each step's first launch
    overlapping the previous step's last); the result must equal n single
    do_step calls bit for bit, across a change of dt0 between calls."""
    import splash_gb300 as sg

    mesh = mesh_of("hex", 4)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=8)
    params = sg.SolverParams(accretion_rate=1e-2, e_acc=0.5, omega_acc_abs=0.5, tilt_angle=0.2,
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    a = sg.Solver(mesh, U0, 5, gam, 0.0, True, params=params, solver=3, precision=sg.PREC_MIXED)
    b = sg.Solver(mesh, U0, 5, gam, 0.0, True, params=params, solver=3, precision=sg.PREC_MIXED)
    a.do_steps(11, 1e-3)
    a.do_steps(6, 5e-4)
    for _ in range(11):
        b.do_step(1e-3)
    for _ in range(6):
        b.do_step(5e-4)
    assert np.array_equal(a.get_state(), b.get_state())
    assert a.time() == b.time() and a.last_dt() == b.last_dt()
    a.close()
    b.close()


@pytest.mark.parametrize("field", [0, 4])
def test_nan_input_stop_flag_mixed_like_fp64(field):
    """A NaN planted in the host input state: in the density it reaches the
    fluxes and latches the stop flag (MUSCL_base.hpp:264-268); in the energy
    the pressure floor swallows it (MUSCL_base.hpp:538) and the step does not
    stop.  The mixed path must stop exactly when the FP64 path (and the
    reference) does, and carry the same NaN pattern in its state."""
    from test_gpu_parity import gpu_solver

    c = dict(load("state_hex3_hllc_acc.npz"))
    U = c["U0"].copy()
    U[5, field] = np.nan
    out = {}
    for prec in (0, 1):
        s = gpu_solver(c, precision=prec)
        s.set_state(U)
        s.do_step(1e-3)
        out[prec] = (s.get_stop_check(), np.isnan(s.get_state()))
    assert out[0][0] == out[1][0] == (field == 0)
    if field == 4:
        assert np.array_equal(out[0][1], out[1][1])


def test_mixed_quad7_shear_close_to_fp64():
    """quad_sphere(7) (98,304 faces, four slots per face: the 4-slot update
    launches), MUSCL_HLLC, the shear layer of seed 2, 200 steps of dt0 = 1e-4:
    the mixed state against the FP64 state, relative L1 per field."""
    import splash_gb300 as sg

    mesh = mesh_of("quad", 7)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.shear_layer(g.unit_face_centers(), gam, seed=2)
    a = sg.MUSCL_HLLC(mesh, U0, 5, gam, 0.0, False)
    b = sg.MUSCL_HLLC(mesh, U0, 5, gam, 0.0, False, precision=sg.PREC_MIXED)
    a.do_steps(200, 1e-4)
    b.do_steps(200, 1e-4)
    Ua, Ub = a.get_state(), b.get_state()
    area = g["area"][:, None]
    l1 = np.sum(area * np.abs(Ub - Ua), axis=0) / np.sum(area * np.abs(Ua), axis=0)
    assert l1[0] < 1e-6 and l1[4] < 1e-6, l1
    assert np.all(l1[1:4] < 1e-5), l1
    assert abs(b.time() - a.time()) <= 1e-6 * a.time()
    assert a.get_stop_check() == b.get_stop_check()
