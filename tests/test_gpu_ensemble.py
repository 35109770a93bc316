"""Ensembles: every member advanced by the shared batched launches must
compute exactly what a standalone mixed-precision solver computes (same
kernels, same per-face arithmetic), whatever block schedule the autotuner
picked.  Members mix the adiabatic solvers (dim 5) and the isothermal one
(dim 4) in the same launches."""
import numpy as np
import pytest

from helpers import mesh_of

pytestmark = pytest.mark.gpu


def members(seed=7, count=10):
    import splash_gb300 as sg

    rng = np.random.default_rng(seed)
    specs = [("hex", 3)] * 4 + [("hex", 4)] * 3 + [("quad", 3)] * 2 + [("hex", 5)]
    out = []
    gam = sg.initial_conditions.gam2d(4 / 3)
    for i, (kind, level) in enumerate(specs[:count]):
        mesh = mesh_of(kind, level)
        r = sg.Geometry(mesh).unit_face_centers()
        U = (sg.initial_conditions.rotating_blob(r, gam, seed=100 + i) if i % 2 == 0
             else sg.initial_conditions.quiet_noise(r, gam, seed=100 + i))
        params = sg.SolverParams(accretion_rate=float(10 ** rng.uniform(-4, -1)), e_acc=0.5,
                                 omega_acc_abs=float(rng.uniform(0, 1)),
                                 tilt_angle=float(rng.uniform(0, np.pi / 2)), acc_width=0.1,
                                 alpha=1e-6, friction_on=bool(i % 3))
        solver = [1, 2, 3][i % 3]
        if i % 4 == 1:  # isothermal members: 4 state fields, no source
            solver, U = sg.SOLVER_HLLE, np.ascontiguousarray(U[:, :4])
        out.append({"mesh": mesh, "U_in": U, "gam": gam, "omega_ns": 0.0, "accretion_on": True,
                    "params": params, "solver": solver})
    return out


def test_ensemble_members_equal_standalone_solvers():
    import splash_gb300 as sg

    ms = members()
    ens = sg.Ensemble(ms, autotune=True)
    n, total = ens.size()
    assert n == len(ms) and total == sum(m["U_in"].shape[0] for m in ms)
    sched = ens.schedule()
    assert sched["recon_width"] in (32, 64, 128)
    assert all(t > 0 for row in sched["trial_ms"] for t in row)
    ens.do_steps(25, 1e-2)  # dt0 large: every member takes its own CFL dt
    dts = set()
    for i, m in enumerate(ms):
        s = sg.Solver(m["mesh"], m["U_in"], m["U_in"].shape[1], m["gam"], 0.0, True, params=m["params"],
                      solver=m["solver"], precision=sg.PREC_MIXED)
        s.do_steps(25, 1e-2)
        info = ens.member_info(i)
        assert np.array_equal(ens.get_state(i), s.get_state()), i
        assert info["t"] == s.time() and info["dt"] == s.last_dt()
        assert info["err"] == s.error_word()
        dts.add(info["dt"])
        s.close()
    assert len(dts) > 1  # members really advance with different dt


def test_ensemble_schedule_does_not_change_results():
    import splash_gb300 as sg

    ms = members(seed=3, count=6)
    a = sg.Ensemble(ms, autotune=False)
    b = sg.Ensemble(ms, autotune=True)
    a.do_steps(10, 1e-3)
    b.do_steps(10, 1e-3)
    for i in range(len(ms)):
        assert np.array_equal(a.get_state(i), b.get_state(i))


def test_batched_and_single_runs_repeat_bit_for_bit():
    """The step's kernels overlap their predecessors (programmatic dependent
    launch); on small meshes whole grids are resident at once, so a state
    read that bypassed the predecessor's writes would show here as
    run-to-run differences."""
    import splash_gb300 as sg

    ms = members(seed=11)
    runs = []
    for _ in range(3):
        e = sg.Ensemble(ms, autotune=False)
        e.do_steps(30, 1e-2)
        runs.append([e.get_state(i) for i in range(len(ms))])
        e.close()
    for r in runs[1:]:
        assert all(np.array_equal(x, y) for x, y in zip(runs[0], r))
    m = ms[0]
    single = []
    for _ in range(3):
        s = sg.Solver(m["mesh"], m["U_in"], m["U_in"].shape[1], m["gam"], 0.0, True, params=m["params"],
                      solver=m["solver"], precision=sg.PREC_MIXED)
        s.do_steps(30, 1e-2)
        single.append(s.get_state())
        s.close()
    assert all(np.array_equal(single[0], x) for x in single[1:])
    assert np.array_equal(single[0], runs[0][0])


def test_batched_workload_members_match_oracle():
    """Members of the 512-member batched workload (splash_gb300.workloads,
    seed 3) against the FP64 oracle run per member with the member's own
    accretion parameters and CFL dt: the three members that latch a stop
    (181, 187, 437: negative extra dt, physics/adiabatic.hpp:573-577, as
    accreted matter spins up past sqrt(GM)) and a seeded sample of the
    members on hex(3..5), dims 4 and 5.  503 steps (the benchmark's 3 + 500):
    the stop bits equal the oracle's, each latching within one step of the
    oracle's, the relative L1 density error of the mixed path is below 1e-5,
    and the simulated times agree to 1e-6."""
    import splash_gb300 as sg
    from splash_gb300 import workloads

    from helpers import make_oracle

    draws = workloads.ensemble_draws(512, 3)
    rng = np.random.default_rng(3)
    small = [d["index"] for d in draws if d["level"] <= 5 and d["index"] not in (181, 187, 437)]
    pick = [181, 187, 437] + sorted(int(i) for i in rng.choice(small, size=9, replace=False))
    sub = [draws[i] for i in pick]
    centres, geoms = {}, {}
    for d in sub:
        if d["level"] not in geoms:
            geoms[d["level"]] = sg.Geometry(sg.icosphere_hex(d["level"]))
            centres[d["level"]] = geoms[d["level"]].unit_face_centers()
    members = workloads.ensemble_members(sg, sub, centres)
    ens = sg.Ensemble(members, autotune=False)
    steps = 503
    first = [None] * len(sub)
    for k in range(steps):
        ens.do_steps(1, 1.0)
        for i in range(len(sub)):
            if first[i] is None and ens.member_info(i)["err"]:
                first[i] = k + 1
    for i, (d, m) in enumerate(zip(sub, members)):
        o = make_oracle(geoms[d["level"]], {"U0": m["U_in"], "gam": m["gam"], "accretion_on": True,
                                            "params": np.array(m["params"].as_list()),
                                            "solver": m["solver"]}, dim=d["dim"])
        bits, o_first = 0, None
        for k in range(steps):
            b = o.do_step(1.0)
            if b and o_first is None:
                o_first = k + 1
            bits |= b
        info = ens.member_info(i)
        assert info["err"] == bits, (d["index"], info["err"], bits)
        if bits:
            assert abs(first[i] - o_first) <= 1, (d["index"], first[i], o_first)
        U, R = ens.get_state(i), o.get_state()
        area = geoms[d["level"]]["area"]
        l1 = np.sum(area * np.abs(U[:, 0] - R[:, 0])) / np.sum(area * np.abs(R[:, 0]))
        assert l1 < 1e-5, (d["index"], l1)
        assert abs(info["t"] - o.info()["t"]) <= 1e-6 * o.info()["t"], (d["index"], info["t"], o.info()["t"])
    assert sum(1 for i in range(len(sub)) if ens.member_info(i)["err"]) == 3
    ens.close()


@pytest.mark.parametrize("order", [0, 1, 2])
def test_persistent_launch_equals_standalone_solvers(order):
    """The persistent schedule (one cooperative launch per do_steps call,
    grid barriers between the phases) computes exactly what the standalone
    mixed solvers compute, for every tile order; 25 steps in one launch
    equal five launches of 5 steps and the five-launch schedule."""
    import splash_gb300 as sg

    ms = members(seed=13)
    ens = sg.Ensemble(ms, autotune=False)
    ens.set_schedule(order, 0)
    assert ens.schedule()["persistent"]
    ens.do_steps(25, 1e-2)
    ens.synchronize()
    for i, m in enumerate(ms):
        s = sg.Solver(m["mesh"], m["U_in"], m["U_in"].shape[1], m["gam"], 0.0, True, params=m["params"],
                      solver=m["solver"], precision=sg.PREC_MIXED)
        s.do_steps(25, 1e-2)
        info = ens.member_info(i)
        assert np.array_equal(ens.get_state(i), s.get_state()), (order, i)
        assert info["t"] == s.time() and info["dt"] == s.last_dt() and info["err"] == s.error_word()
        s.close()
    pieces = sg.Ensemble(ms, autotune=False)
    pieces.set_schedule(order, 0)
    for _ in range(5):
        pieces.do_steps(5, 1e-2)
    five = sg.Ensemble(ms, autotune=False)
    five.set_schedule(order, 64)
    assert not five.schedule()["persistent"]
    five.do_steps(25, 1e-2)
    for i in range(len(ms)):
        assert np.array_equal(pieces.get_state(i), ens.get_state(i))
        assert np.array_equal(five.get_state(i), ens.get_state(i))
    for e in (ens, pieces, five):
        e.close()


def test_full_batched_workload_matches_oracle_record():
    """All 512 members of the batched workload (503 steps, own CFL dt)
    against the oracle's record (tests/golden/ensemble_oracle_c3.json, made
    by gen_ensemble_oracle.py: every member run on the FP64 oracle): every
    member's stop bits equal the oracle's, each latched within one step of
    the oracle's first, the times agree to 1e-6 and the total mass (energy)
    to 1e-7 (1e-6) relative."""
    import json

    import splash_gb300 as sg
    from splash_gb300 import workloads

    from helpers import GOLDEN

    rec = json.loads((GOLDEN / "ensemble_oracle_c3.json").read_text())
    draws = workloads.ensemble_draws(512, 3)
    members = workloads.ensemble_members(sg, draws)
    ens = sg.Ensemble(members, autotune=False)
    first = [None] * len(draws)
    for k in range(rec["steps"]):
        ens.do_steps(1, rec["dt0"])
        if k >= 400:  # the recorded latches come late in the run
            for r in rec["members"]:
                i = r["index"]
                if r["bits"] and first[i] is None and ens.member_info(i)["err"]:
                    first[i] = k + 1
    geoms = {}
    for r in rec["members"]:
        i = r["index"]
        info = ens.member_info(i)
        assert info["err"] == r["bits"], (i, info["err"], r["bits"])
        for bit, step in r["first_step"].items():
            assert first[i] is not None and abs(first[i] - step) <= 1, (i, first[i], step)
        assert abs(info["t"] - r["t"]) <= 1e-6 * r["t"], (i, info["t"], r["t"])
        lv = r["level"]
        if lv not in geoms:
            geoms[lv] = sg.Geometry(sg.icosphere_hex(lv))["area"]
        U = ens.get_state(i)
        mass = float(np.sum(geoms[lv] * U[:, 0]))
        assert abs(mass - r["mass"]) <= 1e-7 * abs(r["mass"]), (i, mass, r["mass"])
        if r["dim"] == 5:
            en = float(np.sum(geoms[lv] * U[:, 4]))
            assert abs(en - r["energy"]) <= 1e-6 * abs(r["energy"]), (i, en, r["energy"])
    assert sum(1 for r in rec["members"] if r["bits"]) == 3
    ens.close()
