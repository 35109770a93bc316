"""The CPU oracle (oracle/splash_oracle.cpp) pinned against the reference:
per-function known answers and multi-step states produced by running the
reference solver itself (tests/golden/gen_golden.py).  On x86-64 both are
the same compiler and libm without FMA, so agreement is bit-for-bit."""
import numpy as np
import pytest

from helpers import BIT_EXACT_HOST, load, make_oracle, mesh_of, rel_linf

FUNC_CASES = ["hllep", "hllc", "hllcp", "hllcp_nofric"]
STATE_CASES = ["c0_hex4_hllep", "c1_hex4_hllcp", "hex3_hllc_acc", "hex3_hllcp_acc",
               "hex3_hllcp_nofric", "quad3_hllc_acc", "shear_quad4_hllc"]


def _same(a, b, rtol=1e-13):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if BIT_EXACT_HOST:
        both_nan = np.isnan(a) & np.isnan(b)
        return bool(np.all((a.view(np.uint64) == b.view(np.uint64)) | both_nan))
    return bool(np.allclose(a, b, rtol=rtol, atol=0, equal_nan=True))


@pytest.fixture(scope="module")
def geoms():
    import splash_gb300 as sg

    return {("hex", 3): sg.Geometry(mesh_of("hex", 3)), ("hex", 4): sg.Geometry(mesh_of("hex", 4)),
            ("quad", 3): sg.Geometry(mesh_of("quad", 3)), ("quad", 4): sg.Geometry(mesh_of("quad", 4))}


@pytest.mark.parametrize("case", FUNC_CASES)
def test_functions_known_answers(case, geoms):
    f = load(f"funcs_{case}.npz")
    g = geoms[(str(f["mesh"]), int(f["level"]))]
    nf = g.n_faces
    o = make_oracle(g, {"U0": np.ones((nf, 5)), "gam": f["gam"], "accretion_on": f["accretion_on"],
                        "params": f["params"], "solver": f["solver"]})
    for i in range(len(f["face"])):
        face, edge = int(f["face"][i]), int(f["edge"][i])
        F, _ = o.flux_star(f["ul"][i], f["ur"][i], face, edge)
        assert _same(F, f["F"][i]), (case, "flux_star", i, F, f["F"][i])
        lim = o.limiter(f["r"][i], f["w"][i], face, edge, float(f["dt"]))
        assert _same(lim, f["lim"][i]), (case, "limiter", i, f["r"][i], lim, f["lim"][i])
        src = o.source(f["uc"][i], face)
        assert _same(src, f["src"][i]), (case, "source", i, src, f["src"][i])


@pytest.mark.parametrize("case", ["hlle_hex3", "hlle_quad3"])
def test_isothermal_functions_known_answers(case, geoms):
    """The isothermal solver's defined functions (flux, char_vel, HLLE
    flux_star; MUSCL_HLLE, dim 4) against the reference's own outputs."""
    f = load(f"isofuncs_{case}.npz")
    g = geoms[(str(f["mesh"]), int(f["level"]))]
    o = make_oracle(g, {"U0": np.ones((g.n_faces, 4)), "gam": f["gam"], "accretion_on": False,
                        "params": np.array([0, 0, 0, 0, 0.1, 1e-6, 1.0]), "solver": 4}, dim=4)
    kinds = set()
    for i in range(len(f["face"])):
        face, edge = int(f["face"][i]), int(f["edge"][i])
        fl = o.iso_flux(f["ul"][i], face, edge)
        assert _same(fl, f["fl"][i]), (case, "flux", i, fl, f["fl"][i])
        cv = o.iso_char_vel(f["ul"][i], f["ur"][i], face, edge)
        assert _same(cv, f["cv"][i]), (case, "char_vel", i, cv, f["cv"][i])
        F, _ = o.flux_star(f["ul"][i], f["ur"][i], face, edge)
        assert _same(F, f["F"][i]), (case, "flux_star", i, F, f["F"][i])
        kinds.add("left" if cv[0] >= 0 else ("right" if cv[1] <= 0 else "star"))
    assert kinds == {"left", "right", "star"}, kinds


@pytest.mark.parametrize("case", STATE_CASES)
def test_states_match_reference(case, geoms):
    c = load(f"state_{case}.npz")
    g = geoms[(str(c["mesh"]), int(c["level"]))]
    o = make_oracle(g, c)
    done = 0
    for k, nstep in enumerate(c["steps"]):
        bits = o.do_steps(int(nstep) - done, float(c["dt0"]))
        done = int(nstep)
        info = o.info()
        U = o.get_state()
        assert info["steps"] == nstep
        assert bool(info["stop"]) == bool(c["stop"][k]), (case, nstep)
        assert _same(info["dt"], c["dt"][k]), (case, nstep, info["dt"], c["dt"][k])
        assert _same(info["t"], c["t"][k]), (case, nstep)
        if BIT_EXACT_HOST:
            assert _same(U, c["U"][k]), (case, nstep, rel_linf(U, c["U"][k]))
        else:
            assert np.all(rel_linf(U, c["U"][k]) < 1e-10), (case, nstep)


def test_mid_size_workload_matches_reference():
    """The accreting mid-size workload (icosphere_hex(7), 163,842 faces, HLLC+,
    quiet noise of seed 1, dt0 = 2e-4) after 100 steps, against the
    reference's own state on every 61st face and its per-field sums over all
    faces."""
    import hashlib

    import splash_gb300 as sg

    c = load("state_c1_hex7_hllcp.npz")
    g = sg.Geometry(mesh_of(str(c["mesh"]), int(c["level"])))
    U0 = sg.initial_conditions.quiet_noise(g.unit_face_centers(), float(c["gam"]), seed=int(c["seed"]))
    assert hashlib.sha256(np.ascontiguousarray(U0, "<f8").tobytes()).hexdigest() == str(c["U0_sha256"])
    case = {k: c[k] for k in ("gam", "accretion_on", "solver", "params")}
    case["U0"] = U0
    o = make_oracle(g, case)
    o.do_steps(int(c["steps"]), float(c["dt0"]))
    info, U = o.info(), o.get_state()
    assert bool(info["stop"]) == bool(c["stop"])
    assert _same(info["dt"], c["dt"]) and _same(info["t"], c["t"])
    assert _same(U[c["index"]], c["U_subset"])
    assert np.allclose(U.sum(axis=0), c["U_sum"], rtol=1e-12, atol=0)


def test_oracle_thread_count_invariance(geoms):
    """The reference is bit-identical across OpenMP thread counts; so is the oracle."""
    c = load("state_hex3_hllcp_acc.npz")
    g = geoms[("hex", 3)]
    outs = []
    for th in (1, 3, 8):
        o = make_oracle(g, c, threads=th)
        o.do_steps(5, float(c["dt0"]))
        outs.append(o.get_state())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_planted_limiter_mistake_is_caught(geoms):
    """The known-answer comparison is sensitive: a perturbed ratio changes
    the limiter output (the mistake is planted in the oracle input, on CPU)."""
    f = load("funcs_hllcp.npz")
    g = geoms[("hex", 3)]
    o = make_oracle(g, {"U0": np.ones((g.n_faces, 5)), "gam": f["gam"],
                        "accretion_on": f["accretion_on"], "params": f["params"],
                        "solver": f["solver"]})
    i, k = next((i, k) for i in range(len(f["face"])) for k in range(5)
                if 0.05 < f["r"][i][k] < 0.95)
    r = f["r"][i].copy()
    r[k] *= 1 + 1e-9
    lim = o.limiter(r, f["w"][i], int(f["face"][i]), int(f["edge"][i]), float(f["dt"]))
    assert not _same(lim, f["lim"][i])
