"""The reference's initial-condition recipes (make_input.py) restated without
pandas (splash_gb300.input_recipes), against the arrays the reference's own
functions wrote on the same face centres (tests/golden/gen_ic_golden.py),
and the results/final_state.dat restart path (test.cpp:34-35,
physics/adiabatic.hpp:335-348)."""
import numpy as np
import pytest

from helpers import load, mesh_of


@pytest.mark.parametrize("mesh", ["hex3", "quad3"])
def test_recipes_match_reference(mesh, tmp_path):
    import splash_gb300 as sg
    from splash_gb300 import input_recipes as ir

    ref = load(f"ic_recipes_{mesh}.npz")
    kind, level = mesh[:-1], int(mesh[-1])
    text = ir.format_face_centers(sg.Geometry(mesh_of(kind, level)).unit_face_centers())
    assert text == str(ref["face_centers_text"])
    (tmp_path / "face_centers.dat").write_text(text)
    fc = ir.read_face_centers(tmp_path / "face_centers.dat")
    for name, recipe in ir.RECIPES.items():
        U = recipe(fc)
        R = ref[name]
        assert U.shape == R.shape, name
        assert np.array_equal(U.view(np.uint64), R.view(np.uint64)), (name, np.max(np.abs(U - R)))
        assert (ir.RECIPE_FLOAT_FORMAT.get(name) or "") == str(ref[name + "__float_format"]), name


def test_input_dat_text_and_reader():
    """The writer's text reads back through the reference's reader rule
    (whitespace-separated values, row-major) to the written values: exactly
    at full precision, to the format's rounding with "%.15f"."""
    import splash_gb300 as sg
    from splash_gb300 import input_recipes as ir

    g = sg.Geometry(mesh_of("hex", 3))
    fcs = g.unit_face_centers()
    U = ir.make_input_5_sp_layer(fcs)
    full = ir.format_input_dat(U)
    back = np.array(full.split(), dtype=np.float64).reshape(U.shape)
    assert np.array_equal(back, U)
    fixed = ir.format_input_dat(U, "%.15f")
    back = np.array(fixed.split(), dtype=np.float64).reshape(U.shape)
    assert np.all(np.abs(back - U) <= 5e-16)
    assert all(len(v.split(".")[1]) == 15 for v in fixed.split()[:10])


def test_final_state_restart_round_trip(tmp_path):
    """write_final_state prints the state with the C++ stream defaults (six
    significant digits, adiabatic.hpp:335-348); the reference restarts by
    reading that file in place of input/input.dat (test.cpp:35).  Reading it
    back, setting it as the state and writing it again gives the same text,
    and a solver restarted from the file computes exactly what one created
    from the parsed values computes (CPU side: the oracle)."""
    import splash_gb300 as sg
    from helpers import make_oracle

    g = sg.Geometry(mesh_of("hex", 3))
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), gam, seed=9)
    case = {"U0": U0, "gam": gam, "accretion_on": True, "solver": 3,
            "params": np.array([1e-2, 0.5, 0.5, 0.2, 0.1, 1e-6, 1.0])}
    o = make_oracle(g, case)
    o.do_steps(5, 1e-3)
    text = sg.format_final_state(o.get_state())
    # the C++ default stream format: %g with 6 significant digits, a space after each value
    first = o.get_state()[0]
    assert text.splitlines()[0] == "".join(f"{x:g} " for x in first)
    path = tmp_path / "final_state.dat"
    path.write_text(text)
    U_re = sg.read_input_dat(path, g.n_faces, 5)
    assert sg.format_final_state(U_re) == text
    a = make_oracle(g, dict(case, U0=U_re))
    b = make_oracle(g, dict(case, U0=np.array(text.split(), dtype=np.float64).reshape(-1, 5)))
    a.do_steps(3, 1e-3)
    b.do_steps(3, 1e-3)
    assert np.array_equal(a.get_state(), b.get_state())


@pytest.mark.gpu
def test_solver_restart_from_final_state(tmp_path):
    """Through the C ABI: the solver's results/final_state.dat is the text of
    the reference's writer; a solver restarted from it (time from 0, as in
    the reference) writes the same file back and then steps like the oracle
    started from the parsed values (1e-10 relative L-infinity per field)."""
    import splash_gb300 as sg
    from helpers import make_oracle, rel_linf

    mesh = mesh_of("hex", 4)
    g = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.input_recipes.make_input_5_cos_bell(g.unit_face_centers())
    params = sg.SolverParams(accretion_rate=1e-2, e_acc=0.5, omega_acc_abs=0.5, tilt_angle=0.2,
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    s = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, True, params=params)
    s.do_steps(5, 1e-3)
    path = tmp_path / "final_state.dat"
    s.write_final_state(path)
    text = path.read_text()
    assert text == sg.format_final_state(s.get_state())
    U_re = sg.read_final_state(path, g.n_faces, 5)
    r = sg.MUSCL_HLLCplus(mesh, U_re, 5, gam, 0.0, True, params=params)
    assert r.time() == 0.0
    r.write_final_state(tmp_path / "again.dat")
    assert (tmp_path / "again.dat").read_text() == text
    r.do_steps(3, 1e-3)
    o = make_oracle(g, {"U0": U_re, "gam": gam, "accretion_on": True, "solver": 3,
                        "params": np.array(params.as_list())})
    o.do_steps(3, 1e-3)
    assert np.all(rel_linf(r.get_state(), o.get_state()) < 1e-10)
