"""GPU isothermal solver (MUSCL_HLLE, dim 4) through the C ABI against the
CPU oracle's restatement of it.

The reference's isothermal flux, char_vel and HLLE flux_star are pinned by
the reference's own outputs (tests/test_oracle.py); its limiter and step are
undefined behaviour in the reference (a fifth state field and an
uninitialised limiter variable), so the step itself is compared with the
oracle's defined restatement: parity unpinned against the reference.  Both
sides use the reference's operation order with IEEE divisions and no
transcendental, so the states must agree bit for bit."""
import numpy as np
import pytest

from helpers import make_oracle, mesh_of, rel_linf

pytestmark = pytest.mark.gpu

GAM = 2 - 1 / (4 / 3)


def _state(g, recipe, seed):
    import splash_gb300 as sg

    r = g.unit_face_centers()
    f = {"blob": sg.initial_conditions.rotating_blob, "shear": sg.initial_conditions.shear_layer,
         "quiet": sg.initial_conditions.quiet_noise}[recipe]
    return np.ascontiguousarray(f(r, GAM, seed=seed)[:, :4])


@pytest.mark.parametrize("kind,level,recipe,seed,dt0", [("hex", 4, "blob", 0, 1e-3), ("quad", 4, "shear", 2, 1e-3),
                                                        ("hex", 3, "quiet", 1, 1e-3), ("hex", 3, "blob", 5, 1.0)])
def test_isothermal_matches_oracle(kind, level, recipe, seed, dt0):
    import splash_gb300 as sg

    mesh = mesh_of(kind, level)
    g = sg.Geometry(mesh)
    U0 = _state(g, recipe, seed)
    s = sg.MUSCL_HLLE(mesh, U0, 4, GAM)
    o = make_oracle(g, {"U0": U0, "gam": GAM, "accretion_on": False,
                        "params": np.array([0, 0, 0, 0, 0.1, 1e-6, 1.0]), "solver": 4}, dim=4)
    done = 0
    for n in (1, 9, 30):
        s.do_steps(n - done, dt0)
        o.do_steps(n - done, dt0)
        done = n
        U, Uo = s.get_state(), o.get_state()
        info = o.info()
        assert U.shape == (g.n_faces, 4)
        assert np.array_equal(U, Uo), (kind, level, recipe, n, rel_linf(U, Uo))
        assert s.last_dt() == info["dt"] and s.time() == info["t"]
        assert s.get_stop_check() == info["stop"]
    if dt0 == 1.0:  # the CFL clip 0.1 h0 / max(|v|, a) decides dt
        assert s.last_dt() < 0.1 * g.h0 * 1.0000001


def test_isothermal_writers(tmp_path):
    import splash_gb300 as sg

    mesh = mesh_of("hex", 3)
    g = sg.Geometry(mesh)
    U0 = _state(g, "blob", 3)
    s = sg.MUSCL_HLLE(mesh, U0, 4, GAM)
    s.do_steps(5, 1e-3)
    U = s.get_state()
    p = tmp_path / "p.dat"
    s.write_t_p(p)
    vals = np.array(p.read_text().split(), dtype=float)
    # time, then a^2 Sigma per face (default stream precision: 6 digits)
    assert np.allclose(vals[1:], U[:, 0], rtol=1e-5)
    s.write_t_omega_z(tmp_path / "om.dat")
    s.write_t_curl(tmp_path / "curl.dat")
    assert len((tmp_path / "om.dat").read_text().split()) == g.n_faces + 1
    with pytest.raises(sg.SplashError):
        s.get_light_curves()  # the isothermal class has none
    assert s.diagnostics()[4] == 0.0


def test_isothermal_mixed_close_to_fp64():
    """FP32 reconstruction and HLLE fluxes with the FP64 state, against the
    FP64 isothermal path: shear layer on quad(5), 300 steps."""
    import splash_gb300 as sg

    mesh = mesh_of("quad", 5)
    g = sg.Geometry(mesh)
    U0 = _state(g, "shear", 2)
    a = sg.MUSCL_HLLE(mesh, U0, 4, GAM)
    b = sg.MUSCL_HLLE(mesh, U0, 4, GAM, precision=sg.PREC_MIXED)
    a.do_steps(300, 1e-3)
    b.do_steps(300, 1e-3)
    Ua, Ub = a.get_state(), b.get_state()
    area = g["area"]
    l1 = np.sum(area * np.abs(Ub[:, 0] - Ua[:, 0])) / np.sum(area * np.abs(Ua[:, 0]))
    assert l1 < 1e-5, l1
    mom = np.sum(area[:, None] * np.abs(Ub[:, 1:] - Ua[:, 1:])) / np.sum(area[:, None] * np.abs(Ua[:, 1:]))
    assert mom < 1e-4, mom
    assert abs(b.time() - a.time()) <= 1e-6 * a.time()
    assert not a.get_stop_check() and not b.get_stop_check()


def test_isothermal_mixed_hex7_close_to_fp64():
    """The isothermal solver on icosphere_hex(7), whose update grid (1,281
    blocks of 128) is about one wave on a 152-SM GB300: the mixed path runs
    its early-state update launches there.  Rotating blob, 50 steps, against
    the FP64 isothermal path."""
    import splash_gb300 as sg

    mesh = mesh_of("hex", 7)
    g = sg.Geometry(mesh)
    U0 = _state(g, "blob", 7)
    a = sg.MUSCL_HLLE(mesh, U0, 4, GAM)
    b = sg.MUSCL_HLLE(mesh, U0, 4, GAM, precision=sg.PREC_MIXED)
    a.do_steps(50, 1e-3)
    b.do_steps(50, 1e-3)
    Ua, Ub = a.get_state(), b.get_state()
    area = g["area"]
    l1 = np.sum(area * np.abs(Ub[:, 0] - Ua[:, 0])) / np.sum(area * np.abs(Ua[:, 0]))
    assert l1 < 1e-6, l1
    assert abs(b.time() - a.time()) <= 1e-6 * a.time()
    assert not a.get_stop_check() and not b.get_stop_check()
