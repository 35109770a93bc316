"""Gradient check of the discrete adjoint on the adjoint workload.

Workload: icosphere_hex(6) (40,962 faces), MUSCL_HLLC, dim 5, gam3d 4/3,
FP64, 1000 steps at dt0 = 5e-4, checkpoints every 50 steps.  Initial state:
the rotating-blob recipe of the small plain-method workload with seed 4.
Accretion on (e_acc 0.5, omega_acc_abs 0.5, acc_width 0.1, friction on,
alpha 1e-6).  Target Sigma*: a forward run with accretion_rate 2e-2 and
tilt_angle 0.3 rad.  Loss: 1/2 sum_n area_n (Sigma_n - Sigma*_n)^2, its
gradient taken at accretion_rate 1e-2, tilt_angle 0.1 rad with respect to
U0 (all 5 fields per face) and theta = (accretion_rate, tilt_angle,
omega_acc_abs).  Along seeded random directions the adjoint's directional
derivative is compared with central finite differences (h = 1e-6, relative
to each component's scale; also a sweep of smaller h) and with the
tangent-linear model; parameter-only directions are checked the same way.

The limited scheme is not differentiable where a field is exactly uniform
(the far field of this initial state, where Sigma and Pi are 1 to the last
bit) and has kinks at grid scale, so along state directions the central
differences approach the derivative only as h shrinks; parameter
directions scale with the source's own profile and stay differentiable.

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

GAM = sg.initial_conditions.gam2d(4 / 3)


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--dt0", type=float, default=5e-4)
    ap.add_argument("--checkpoint-every", type=int, default=50)
    ap.add_argument("--directions", type=int, default=16)
    ap.add_argument("--h", type=float, default=1e-6)
    ap.add_argument("--h-sweep", type=float, nargs="*", default=[1e-7, 1e-8, 1e-9])
    ap.add_argument("--param-directions", type=int, default=5)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--solver", type=int, default=sg.SOLVER_HLLC)
    ap.add_argument("--out", type=str, default=None)
    a = ap.parse_args(argv)

    mesh = sg.icosphere_hex(a.level)
    geo = sg.Geometry(mesh)
    area = geo["area"].copy()
    U0 = sg.initial_conditions.rotating_blob(geo.unit_face_centers(), GAM, seed=a.seed)
    theta = np.array([1e-2, 0.1, 0.5])
    params = sg.SolverParams(accretion_rate=theta[0], e_acc=0.5, omega_acc_abs=theta[2], tilt_angle=theta[1],
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    base = sg.Solver(mesh, U0, 5, GAM, 0.0, True, params=params, solver=a.solver, precision=sg.PREC_FP64)
    adj = sg.Adjoint(base, checkpoint_every=a.checkpoint_every)

    # plain FP64 forward of the same length (graph replay), for the cost ratio
    base.do_steps(3, a.dt0)
    base.synchronize()
    base.set_state(U0)
    t0 = time.perf_counter()
    base.do_steps(a.steps, a.dt0)
    base.synchronize()
    solver_ms = (time.perf_counter() - t0) * 1e3

    target = adj.forward(U0, np.array([2e-2, 0.3, theta[2]]), a.steps, a.dt0)[:, 0].copy()
    target_clipped = adj.info()["clipped_steps"]
    t0 = time.perf_counter()
    loss, gU, gth = adj.run(U0, theta, a.steps, a.dt0, target)
    grad_wall_ms = (time.perf_counter() - t0) * 1e3
    info = adj.info()
    err_word = adj.error_word()
    Uf = adj.forward(U0, theta, a.steps, a.dt0)
    resid = area * (Uf[:, 0] - target)

    rng = np.random.default_rng(a.seed)
    scale = np.maximum(np.abs(U0).max(axis=0), 1e-3)
    tlm_ms = []

    def check(dU, dth, hs):
        g_adj = float(np.sum(gU * dU) + np.dot(gth, dth))
        _, dUt = adj.tlm(U0, theta, dU, dth, a.steps, a.dt0)
        tlm_ms.append(adj.info()["ms_tlm"])
        g_tlm = float(np.sum(resid * dUt[:, 0]))
        row = {"adjoint": g_adj, "tlm": g_tlm, "rel_adj_tlm": abs(g_adj - g_tlm) / abs(g_tlm), "fd": {}}
        for h in hs:
            Lp, _, _ = adj.run(U0 + h * dU, theta + h * dth, a.steps, a.dt0, target)
            Lm, _, _ = adj.run(U0 - h * dU, theta - h * dth, a.steps, a.dt0, target)
            g_fd = (Lp - Lm) / (2 * h)
            row["fd"][f"{h:.0e}"] = {"value": g_fd, "rel_adj_fd": abs(g_adj - g_fd) / abs(g_fd)}
        return row

    # the seeded joint directions (U0 with per-field scales, and theta)
    joint = []
    for _ in range(a.directions):
        dU = rng.normal(size=U0.shape) * scale
        dth = rng.normal(size=3) * np.array([1e-2, 0.1, 0.5])
        joint.append(check(dU, dth, [a.h] + [h for h in a.h_sweep if h != a.h]))
    # parameter-only directions: the unit directions and seeded ones
    param = []
    for dth in [np.array([1e-2, 0, 0]), np.array([0, 0.1, 0]), np.array([0, 0, 0.5])] + \
            [rng.normal(size=3) * np.array([1e-2, 0.1, 0.5]) for _ in range(a.param_directions)]:
        param.append(check(np.zeros_like(U0), dth, [a.h]))
    fwd, bwd = info["ms_forward"], info["ms_backward"]
    out = {
        "workload": f"icosphere_hex({a.level}) {base.n_faces} faces, solver {a.solver}, FP64, {a.steps} steps "
                    f"dt0={a.dt0}, checkpoints every {a.checkpoint_every}",
        "loss": loss,
        "grad_theta": gth.tolist(),
        "grad_U0_norm": float(np.linalg.norm(gU)),
        "clipped_steps": info["clipped_steps"], "target_clipped_steps": target_clipped,
        "dt_min": info["dt_min"], "dt_max": info["dt_max"], "error_word": err_word,
        "joint_directions": joint,
        "parameter_directions": param,
        "max_rel_adj_tlm": max(r["rel_adj_tlm"] for r in joint + param),
        "joint_max_rel_adj_fd_at_h": max(r["fd"][f"{a.h:.0e}"]["rel_adj_fd"] for r in joint) if joint else None,
        "joint_max_rel_adj_fd_best_h": max(min(v["rel_adj_fd"] for v in r["fd"].values()) for r in joint)
        if joint else None,
        "parameter_max_rel_adj_fd_at_h": max(r["fd"][f"{a.h:.0e}"]["rel_adj_fd"] for r in param),
        "ms_forward_checkpointed": fwd, "ms_backward": bwd, "ms_gradient_wall": grad_wall_ms,
        "ms_solver_forward": solver_ms, "ms_tlm_mean": float(np.mean(tlm_ms)) if tlm_ms else None,
        "adjoint_cost_ratio": (fwd + bwd) / solver_ms,
        "backward_over_forward": bwd / fwd,
        "device_bytes": info["device_bytes"],
    }
    s = json.dumps(out, indent=1)
    print(s)
    if a.out:
        Path(a.out).write_text(s)
    return out


if __name__ == "__main__":
    main()
