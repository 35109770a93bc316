"""FP32-mixed vs FP64 on the large-mesh shear-layer workload.

Cases (all with the shear-layer initial state, seed 2: u_phi = 0.5
tanh(latitude / 0.05), Sigma = 1 + 1e-2 x random real Y_lm (l <= 8),
Pi = Sigma^gam2d, gam3d = 4/3; no accretion; do_step(1e-4) with the CFL
clip picking dt):
  hex9_hllcp   icosphere_hex(9), 2,621,442 faces, MUSCL_HLLCplus, dim 5
  quad9_hllc   quad_sphere(9), 1,572,864 faces, MUSCL_HLLC, dim 5
  quad9_hlle   quad_sphere(9), MUSCL_HLLE, dim 4 (isothermal; the first
               four fields of the same state)
For each case both precisions run the same number of steps from the same
state; reported: face-updates/s of each (CUDA events on the solver stream
around the step loop, state resident), the mixed/FP64 ratio, the relative
L1 and L-infinity error per field of the mixed state against the FP64
state, the relative drift of total mass and angular momentum of each run,
the dt of the last step and the stop flags.

Prints one JSON object (``--out`` also writes it to a file).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import splash_gb300 as sg  # noqa: E402

CASES = {
    "hex9_hllcp": (sg.MESH_ICOSPHERE_HEX, 9, sg.SOLVER_HLLCPLUS, 5),
    "quad9_hllc": (sg.MESH_QUAD_SPHERE, 9, sg.SOLVER_HLLC, 5),
    "quad9_hlle": (sg.MESH_QUAD_SPHERE, 9, sg.SOLVER_HLLE, 4),
}


def timed_steps(torch, solver, steps, dt0):
    stream = torch.cuda.ExternalStream(solver.stream())
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    solver.do_steps(steps, dt0)
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / 1e3


def run_case(torch, name, steps, dt0, warmup):
    kind, level, solver_kind, dim = CASES[name]
    mesh = sg.Mesh(kind, level)
    t0 = time.perf_counter()
    geo = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = np.ascontiguousarray(sg.initial_conditions.shear_layer(geo.unit_face_centers(), gam, seed=2)[:, :dim])
    area = geo["area"].copy()
    setup = {"geometry_s": time.perf_counter() - t0}
    out = {"faces": geo.n_faces, "solver": solver_kind, "dim": dim, "steps": steps, "dt0": dt0}
    states = {}
    for prec_name, prec in (("fp64", sg.PREC_FP64), ("mixed", sg.PREC_MIXED)):
        t0 = time.perf_counter()
        s = sg.Solver(mesh, U0, dim, gam, 0.0, False, params=sg.SolverParams(), solver=solver_kind,
                      precision=prec)
        setup[f"create_{prec_name}_s"] = time.perf_counter() - t0
        diag0 = s.diagnostics()
        # warm-up steps on a copy of the state, then restart from U0
        s.do_steps(warmup, dt0)
        s.synchronize()
        s.set_state(U0)
        secs = timed_steps(torch, s, steps, dt0)
        U = s.get_state()
        diag1 = s.diagnostics()
        states[prec_name] = U
        out[prec_name] = {
            "face_updates_per_s": geo.n_faces * steps / secs, "ms_per_step": secs / steps * 1e3,
            "last_dt": s.last_dt(), "stop": s.get_stop_check(), "error_word": s.error_word(),
            "mass_drift": float(diag1[0] / diag0[0] - 1),
            "angular_momentum_drift": float(np.linalg.norm(diag1[1:4] - diag0[1:4]) /
                                            max(np.linalg.norm(diag0[1:4]), 1e-300)),
        }
        s.close()
    a, b = states["fp64"], states["mixed"]
    out["mixed_over_fp64"] = out["mixed"]["face_updates_per_s"] / out["fp64"]["face_updates_per_s"]
    out["l1_rel_per_field"] = (np.sum(area[:, None] * np.abs(b - a), axis=0) /
                               np.maximum(np.sum(area[:, None] * np.abs(a), axis=0), 1e-300)).tolist()
    out["linf_rel_per_field"] = (np.max(np.abs(b - a), axis=0) /
                                 np.maximum(np.max(np.abs(a), axis=0), 1e-300)).tolist()
    out["setup"] = setup
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--cases", nargs="*", default=list(CASES))
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--dt0", type=float, default=1e-4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--out", type=str, default=None)
    a = ap.parse_args(argv)
    import torch

    res = {name: run_case(torch, name, a.steps, a.dt0, a.warmup) for name in a.cases}
    s = json.dumps(res, indent=1)
    print(s)
    if a.out:
        Path(a.out).write_text(s)
    return res


if __name__ == "__main__":
    main()
