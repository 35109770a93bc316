"""Generates the committed golden fixtures from the reference solver itself.

Runs the reference SPLASH solver compiled from its own sources
(oracle/_ref/ref_runner, built by oracle/ref/Makefile from the reference
checkout) in scratch directories laid out like the reference's working
directory (input/parameters.json, input/input.dat, results/), and stores:

* geom_<mesh><n>.npz     full geometry members (geometry/MUSCL_geometry.hpp:23-40)
* geom_hashes.json       SHA-256 of every geometry array for larger meshes
* funcs_<case>.npz       per-function known answers: flux_star, limiter, source
* isofuncs_<case>.npz    isothermal solver (MUSCL_HLLE, dim 4): flux,
                         char_vel and flux_star known answers
* state_<case>.npz       conserved state after selected steps of do_step

Usage:  python tests/golden/gen_golden.py [--ref-root /path/to/reference]
Only needs the reference checkout and a C++ compiler; it is never run by the
test-suite (the fixtures are committed).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "muscl-scheme-on-spherical-mesh-wip_gb300"))
from splash_gb300 import initial_conditions as ic  # noqa: E402

RUNNER = REPO / "oracle" / "_ref" / "ref_runner"
SOLVERS = {"HLLE_p": 1, "HLLC": 2, "HLLCplus": 3}

ACC_PARAMS = dict(accretion_rate=1e-2, e_acc=0.5, omega_acc_abs=0.5, tilt_angle=0.2,
                  acc_width=0.1, alpha=1e-6, friction_on=True)


def params_json(p: dict) -> dict:
    return {"dim": 5, "dt": 1e-3, "t_max": 1e9, "maxstep": 10**9, "skipstep": 100,
            "gam3d": 4 / 3, "omega_ns": 0.0, "threads": 8, "accretion_on": True, **p}


def run(mode, mesh, level, solver, gam, omega_ns, acc, dt, nsteps, dump_every, U, params,
        seed=0, nsamp=0, threads=8, dim=5):
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "input").mkdir()
        (td / "results").mkdir()
        (td / "input" / "parameters.json").write_text(json.dumps(params_json(params)))
        if U is not None:
            ic.write_input_dat(td / "input" / "input.dat", U)
        out = td / "out"
        cmd = [str(RUNNER), mode, mesh, str(level), solver, str(dim), repr(gam), repr(omega_ns),
               "1" if acc else "0", str(threads), repr(dt), str(nsteps), str(dump_every), str(out),
               str(seed), str(nsamp)]
        subprocess.run(cmd, cwd=td, check=True, stdout=subprocess.DEVNULL)
        res = {}
        for suffix in ("_geom.bin", "_states.bin", "_funcs.bin", "_isofuncs.bin", "_scalars.txt"):
            p = Path(str(out) + suffix)
            if p.exists():
                res[suffix] = p.read_bytes()
        return res


def parse_geometry(b: bytes) -> dict:
    pos = 0

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(b, dtype=dt, count=n, offset=pos)
        pos += a.nbytes
        return a

    nv, nf = take("<i8", 2)
    g = {"vertices": take("<f8", 3 * nv).reshape(nv, 3)}
    sizes = take("<i8", nf)
    g["face_off"] = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    ns = int(g["face_off"][-1])
    g["face_vtx"] = take("<i8", ns).astype(np.int32)
    nsz = take("<i8", nf)
    g["nbr_off"] = np.concatenate([[0], np.cumsum(nsz)]).astype(np.int32)
    g["nbr"] = take("<i8", int(nsz.sum())).astype(np.int32)
    esz = take("<i8", nf)
    assert np.array_equal(esz, sizes), "neighbors_edge size differs from face size"
    g["nbr_edge"] = take("<i8", int(esz.sum())).astype(np.int32)
    g["face_centers"] = take("<f8", 3 * nf).reshape(nf, 3)
    g["normals"] = take("<f8", 3 * nf).reshape(nf, 3)
    g["area"] = take("<f8", nf)
    rec = np.dtype([("en", "<f8", 3), ("bm", "<f8"), ("hp", "<f8"), ("hm", "<f8"),
                    ("ffp", "<i8", 2), ("ffm", "<i8", 2), ("bp", "<f8", 2), ("bmn", "<f8", 2)])
    r = np.frombuffer(b, dtype=rec, count=ns, offset=pos)
    pos += r.nbytes
    g["edge_normals"] = np.ascontiguousarray(r["en"])
    g["bm_dist"] = np.ascontiguousarray(r["bm"])
    g["h_plus"] = np.ascontiguousarray(r["hp"])
    g["h_minus"] = np.ascontiguousarray(r["hm"])
    g["ff_plus"] = np.ascontiguousarray(r["ffp"]).astype(np.int32)
    g["ff_minus"] = np.ascontiguousarray(r["ffm"]).astype(np.int32)
    g["beta_plus"] = np.ascontiguousarray(r["bp"])
    g["beta_minus"] = np.ascontiguousarray(r["bmn"])
    g["h0"] = np.float64(take("<f8", 1)[0])
    assert pos == len(b), "trailing bytes in geometry dump"
    return g


def parse_states(b: bytes, nf: int, dim: int = 5) -> list[dict]:
    rec = np.dtype([("t", "<f8"), ("dt", "<f8"), ("stop", "<i8"), ("steps", "<i8"),
                    ("U", "<f8", (nf, dim))])
    a = np.frombuffer(b, dtype=rec)
    return [{"t": x["t"], "dt": x["dt"], "stop": int(x["stop"]), "steps": int(x["steps"]),
             "U": np.array(x["U"])} for x in a]


def parse_funcs(b: bytes) -> dict:
    nsamp, dim = np.frombuffer(b, dtype="<i8", count=2)
    dt = np.frombuffer(b, dtype="<f8", count=1, offset=16)[0]
    rec = np.dtype([("face", "<i8"), ("edge", "<i8"), ("ul", "<f8", dim), ("ur", "<f8", dim),
                    ("uc", "<f8", dim), ("r", "<f8", dim), ("w", "<f8", dim), ("F", "<f8", dim),
                    ("lim", "<f8", dim), ("src", "<f8", dim)])
    a = np.frombuffer(b, dtype=rec, count=int(nsamp), offset=24)
    out = {k: np.array(a[k]) for k in rec.names}
    out["dt"] = np.float64(dt)
    return out


def unit(fc):
    n = np.sqrt((fc[:, 0] * fc[:, 0] + fc[:, 1] * fc[:, 1]) + fc[:, 2] * fc[:, 2])
    return fc / n[:, None]


def geometry(mesh, level):
    res = run("geometry", mesh, level, "HLLCplus", 1.25, 0.0, False, 1e-3, 0, 0, None, ACC_PARAMS)
    g = parse_geometry(res["_geom.bin"])
    ac, tm = map(float, res["_scalars.txt"].split())
    return g, ac, tm


def array_hashes(g: dict) -> dict:
    out = {}
    for k, v in g.items():
        if k == "h0":
            out[k] = float(v).hex()
            continue
        a = np.ascontiguousarray(v)
        a = a.astype("<i4") if a.dtype.kind == "i" else a.astype("<f8")
        out[k] = hashlib.sha256(a.tobytes()).hexdigest()
    return out


def state_case(name, mesh, level, solver, gam, acc, params, dt, nsteps, dump_every, recipe, seed):
    g, _, _ = geometry(mesh, level)
    r = unit(g["face_centers"])
    U0 = recipe(r, gam, seed=seed)
    res = run("run", mesh, level, solver, gam, 0.0, acc, dt, nsteps, dump_every, U0, params)
    st = parse_states(res["_states.bin"], len(g["area"]))
    rec = {"U0": U0, "gam": np.float64(gam), "dt0": np.float64(dt), "solver": SOLVERS[solver],
           "accretion_on": int(acc), "params": np.array([params[k] for k in (
               "accretion_rate", "e_acc", "omega_acc_abs", "tilt_angle", "acc_width", "alpha")]
               + [1.0 if params["friction_on"] else 0.0]),
           "mesh": mesh, "level": level,
           "steps": np.array([s["steps"] for s in st[1:]]),
           "t": np.array([s["t"] for s in st[1:]]),
           "dt": np.array([s["dt"] for s in st[1:]]),
           "stop": np.array([s["stop"] for s in st[1:]]),
           "U": np.stack([s["U"] for s in st[1:]])}
    np.savez_compressed(HERE / f"state_{name}.npz", **rec)
    print(f"state_{name}: steps {rec['steps'].tolist()} dt {rec['dt'][-1]:.6g} stop {rec['stop'].tolist()}")


def state_subset_case(name, mesh, level, solver, gam, acc, params, dt, nsteps, recipe, seed,
                      stride=61):
    """A state run on a mesh too large for a full fixture: the initial state's
    SHA-256 (the test regenerates it from the recipe), the reference's final
    state on every stride-th face (reference order), its per-field sums over
    all faces, and dt, t and the stop flag of the last step."""
    g, _, _ = geometry(mesh, level)
    U0 = recipe(unit(g["face_centers"]), gam, seed=seed)
    res = run("run", mesh, level, solver, gam, 0.0, acc, dt, nsteps, nsteps, U0, params)
    st = parse_states(res["_states.bin"], len(g["area"]))[-1]
    idx = np.arange(0, len(g["area"]), stride, dtype=np.int64)
    rec = {"U0_sha256": hashlib.sha256(np.ascontiguousarray(U0, "<f8").tobytes()).hexdigest(),
           "seed": seed, "gam": np.float64(gam), "dt0": np.float64(dt),
           "solver": SOLVERS[solver], "accretion_on": int(acc), "mesh": mesh, "level": level,
           "params": np.array([params[k] for k in ("accretion_rate", "e_acc", "omega_acc_abs",
                                                   "tilt_angle", "acc_width", "alpha")]
                              + [1.0 if params["friction_on"] else 0.0]),
           "steps": st["steps"], "t": st["t"], "dt": st["dt"], "stop": st["stop"],
           "index": idx, "U_subset": st["U"][idx], "U_sum": st["U"].sum(axis=0),
           "U_absmax": np.abs(st["U"]).max(axis=0)}
    np.savez_compressed(HERE / f"state_{name}.npz", **rec)
    print(f"state_{name}: steps {st['steps']} dt {st['dt']:.6g} stop {st['stop']} "
          f"({len(idx)} of {len(g['area'])} faces kept)")


def funcs_case(name, solver, params, acc=True, mesh="hex", level=3, nsamp=300, seed=11):
    res = run("functions", mesh, level, solver, 1.25, 0.0, acc, 7e-4, 0, 0, None, params,
              seed=seed, nsamp=nsamp)
    f = parse_funcs(res["_funcs.bin"])
    f.update({"solver": SOLVERS[solver], "gam": np.float64(1.25), "accretion_on": int(acc),
              "mesh": mesh, "level": level,
              "params": np.array([params[k] for k in ("accretion_rate", "e_acc", "omega_acc_abs",
                                                      "tilt_angle", "acc_width", "alpha")]
                                 + [1.0 if params["friction_on"] else 0.0])})
    np.savez_compressed(HERE / f"funcs_{name}.npz", **f)
    print(f"funcs_{name}: {nsamp} samples")


def iso_funcs_case(name, mesh="hex", level=3, nsamp=400, seed=13, gam=1.25):
    """Known answers of the isothermal solver's defined functions (flux,
    char_vel, HLLE flux_star) on seeded 4-field states."""
    res = run("iso_functions", mesh, level, "HLLE", gam, 0.0, False, 7e-4, 0, 0, None, ACC_PARAMS,
              seed=seed, nsamp=nsamp, dim=4)
    b = res["_isofuncs.bin"]
    n = int(np.frombuffer(b, dtype="<i8", count=1)[0])
    rec = np.dtype([("face", "<i8"), ("edge", "<i8"), ("ul", "<f8", 4), ("ur", "<f8", 4), ("fl", "<f8", 4),
                    ("cv", "<f8", 2), ("F", "<f8", 4)])
    a = np.frombuffer(b, dtype=rec, count=n, offset=8)
    out = {k: np.array(a[k]) for k in rec.names}
    out.update({"gam": np.float64(gam), "mesh": mesh, "level": level})
    np.savez_compressed(HERE / f"isofuncs_{name}.npz", **out)
    print(f"isofuncs_{name}: {n} samples")


def writers_case(name, mesh, level, solver, gam, acc, params, dt, nsteps, recipe, seed):
    """The reference's own output files (results/*.dat, light curves) for the
    driver sequence of test.cpp:84-149, stored as text."""
    g, _, _ = geometry(mesh, level)
    U0 = recipe(unit(g["face_centers"]), gam, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "input").mkdir()
        (td / "results").mkdir()
        (td / "input" / "parameters.json").write_text(json.dumps(params_json(params)))
        ic.write_input_dat(td / "input" / "input.dat", U0)
        cmd = [str(RUNNER), "writers", mesh, str(level), solver, "5", repr(gam), "0.0",
               "1" if acc else "0", "8", repr(dt), str(nsteps), "0", str(td / "out")]
        res = subprocess.run(cmd, cwd=td, check=True, capture_output=True, text=True)
        files = {p.name: p.read_text() for p in sorted((td / "results").iterdir())}
        files["lightcurves.txt"] = (td / "out_lightcurves.txt").read_text()
        # the reference's per-step line (MUSCL_base.hpp:211-213)
        files["steplog.txt"] = "".join(l + "\n" for l in res.stdout.splitlines() if l.startswith("t= "))
    rec = {"U0": U0, "gam": np.float64(gam), "dt0": np.float64(dt), "steps": nsteps,
           "solver": SOLVERS[solver], "accretion_on": int(acc), "mesh": mesh, "level": level,
           "files": np.array(list(files.keys())), "texts": np.array(list(files.values()))}
    np.savez_compressed(HERE / f"writers_{name}.npz", **rec)
    print(f"writers_{name}: {sorted(files)}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["isothermal", "writers", "large_geometry", "mid_state"],
                    default=None, help="regenerate one group of fixtures only")
    a = ap.parse_args()
    if not RUNNER.exists():
        sys.exit(f"{RUNNER} missing: make -C oracle/ref REF=<reference checkout>")
    if a.only == "mid_state":
        # the accreting mid-size workload itself: icosphere_hex(7), 163,842
        # faces, HLLC+, quiet noise of seed 1, dt0 = 2e-4, 100 steps
        state_subset_case("c1_hex7_hllcp", "hex", 7, "HLLCplus", ic.gam2d(4 / 3), True,
                          ACC_PARAMS, 2e-4, 100,
                          lambda r, g_, seed: ic.quiet_noise(r, g_, seed=seed), 1)
        return
    if a.only == "large_geometry":
        # the large-mesh workloads' geometries (hex(9): 2,621,442 faces, quad(9):
        # 1,572,864), hashed and merged into geom_hashes.json
        path = HERE / "geom_hashes.json"
        data = json.loads(path.read_text())
        for mesh, level in (("hex", 9), ("quad", 9)):
            g, ac, _ = geometry(mesh, level)
            data["hashes"][f"{mesh}{level}"] = array_hashes(g)
            data["scalars"][f"{mesh}{level}"] = {"area_coeff_acc_width_0.1": ac}
            print(f"{mesh}{level}: {len(g['area'])} faces hashed")
        path.write_text(json.dumps(data, indent=1))
        return
    if a.only == "isothermal":
        iso_funcs_case("hlle_hex3")
        iso_funcs_case("hlle_quad3", mesh="quad", seed=17)
        return
    if a.only == "writers":
        writers_case("hex3_hllcp", "hex", 3, "HLLCplus", ic.gam2d(4 / 3), True, ACC_PARAMS, 1e-3, 5,
                     lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 5)
        return
    # geometry: full arrays for small meshes, hashes for larger ones
    scal = {}
    for mesh, level in (("hex", 2), ("hex", 3), ("quad", 3)):
        g, ac, tm = geometry(mesh, level)
        np.savez_compressed(HERE / f"geom_{mesh}{level}.npz", **g)
        scal[f"{mesh}{level}"] = {"area_coeff_acc_width_0.1": ac}
    hashes = {}
    for mesh, level in (("hex", 4), ("hex", 6), ("hex", 7), ("quad", 4), ("quad", 6)):
        g, ac, tm = geometry(mesh, level)
        hashes[f"{mesh}{level}"] = array_hashes(g)
        scal[f"{mesh}{level}"] = {"area_coeff_acc_width_0.1": ac}
    (HERE / "geom_hashes.json").write_text(json.dumps({"hashes": hashes, "scalars": scal}, indent=1))
    print("geometry done")

    nofric = dict(ACC_PARAMS, friction_on=False)
    funcs_case("hllep", "HLLE_p", ACC_PARAMS)
    funcs_case("hllc", "HLLC", ACC_PARAMS)
    funcs_case("hllcp", "HLLCplus", ACC_PARAMS)
    funcs_case("hllcp_nofric", "HLLCplus", nofric)
    iso_funcs_case("hlle_hex3")
    iso_funcs_case("hlle_quad3", mesh="quad", seed=17)

    gam = ic.gam2d(4 / 3)
    # small plain-method workload: hex(4), HLLE_p, accretion off, dt 1e-3, 100 steps
    state_case("c0_hex4_hllep", "hex", 4, "HLLE_p", gam, False, ACC_PARAMS, 1e-3, 100, 100,
               lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 0)
    # accreting recipe of the mid-size workload on a hex(4) mesh, HLLC+
    state_case("c1_hex4_hllcp", "hex", 4, "HLLCplus", gam, True, ACC_PARAMS, 2e-4, 100, 100,
               lambda r, g_, seed: ic.quiet_noise(r, g_, seed=seed), 1)
    state_case("hex3_hllc_acc", "hex", 3, "HLLC", gam, True, ACC_PARAMS, 1e-3, 50, 10,
               lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 5)
    state_case("hex3_hllcp_acc", "hex", 3, "HLLCplus", gam, True, ACC_PARAMS, 1e-3, 50, 10,
               lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 6)
    state_case("hex3_hllcp_nofric", "hex", 3, "HLLCplus", gam, True, nofric, 1e-3, 50, 10,
               lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 7)
    state_case("quad3_hllc_acc", "quad", 3, "HLLC", gam, True, ACC_PARAMS, 1e-3, 50, 10,
               lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 8)
    # shear layer with the CFL clip active (dt0 = 1e-2 is larger than the clip);
    # u_phi = 0.5 makes g_eff < 0, so extra_dt_constr latches stop_check
    state_case("shear_quad4_hllc", "quad", 4, "HLLC", gam, False, ACC_PARAMS, 1e-2, 30, 10,
               lambda r, g_, seed: ic.shear_layer(r, g_, seed=seed), 2)
    writers_case("hex3_hllcp", "hex", 3, "HLLCplus", gam, True, ACC_PARAMS, 1e-3, 5,
                 lambda r, g_, seed: ic.rotating_blob(r, g_, seed=seed), 5)


if __name__ == "__main__":
    main()
