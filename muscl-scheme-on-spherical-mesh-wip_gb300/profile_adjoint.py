"""Runs one gradient (checkpointed forward + backward) of the adjoint
workload at reduced length, for use under a profiler.

    python muscl-scheme-on-spherical-mesh-wip_gb300/profile_adjoint.py \
        --level 6 --steps 20 --checkpoint-every 10

Workload as the adjoint check (icosphere_hex(level), HLLC by default, FP64,
dt0 = 5e-4, rotating-blob initial state seed 4, accretion on); the loss
target is a forward run with accretion_rate 2e-2, tilt_angle 0.3.  With
--tlm, one tangent-linear run follows.  Prints the CUDA-event times of the
forward, backward and TLM runs.
"""
import argparse
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import splash_gb300 as sg  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--solver", type=int, default=2, choices=[1, 2, 3])
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--checkpoint-every", type=int, default=10)
    ap.add_argument("--tlm", action="store_true")
    a = ap.parse_args()
    gam = sg.initial_conditions.gam2d(4 / 3)
    mesh = sg.icosphere_hex(a.level)
    geo = sg.Geometry(mesh)
    U0 = sg.initial_conditions.rotating_blob(geo.unit_face_centers(), gam, seed=4)
    theta = np.array([1e-2, 0.1, 0.5])
    params = sg.SolverParams(accretion_rate=theta[0], e_acc=0.5, omega_acc_abs=theta[2], tilt_angle=theta[1],
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    base = sg.Solver(mesh, U0, 5, gam, 0.0, True, params=params, solver=a.solver, precision=sg.PREC_FP64)
    adj = sg.Adjoint(base, checkpoint_every=a.checkpoint_every)
    target = adj.forward(U0, np.array([2e-2, 0.3, 0.5]), a.steps, 5e-4)[:, 0].copy()
    loss, _, gth = adj.run(U0, theta, a.steps, 5e-4, target)
    info = adj.info()
    print(f"hex({a.level}) F={base.n_faces} solver={a.solver}: {a.steps} steps, K={a.checkpoint_every}: "
          f"forward {info['ms_forward']:.2f} ms, backward {info['ms_backward']:.2f} ms, loss {loss:.6e}, "
          f"grad_theta {gth}")
    if a.tlm:
        rng = np.random.default_rng(0)
        adj.tlm(U0, theta, rng.normal(size=U0.shape), None, a.steps, 5e-4)
        print(f"tlm {adj.info()['ms_tlm']:.2f} ms")


if __name__ == "__main__":
    main()
