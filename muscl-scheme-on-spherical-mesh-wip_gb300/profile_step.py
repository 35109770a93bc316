"""Runs a few do_step calls of one configuration, for use under a profiler.

    python muscl-scheme-on-spherical-mesh-wip_gb300/profile_step.py \
        --mesh hex --level 7 --solver 3 --precision mixed --steps 5

Builds the solver (geometry, upload, graph capture), then launches `steps`
graph replays of do_step(dt0) and synchronises.  Initial state: Sigma = Pi =
1 with 1e-3 noise (seed 1), accretion on with the mid-size workload's
parameters unless --no-accretion.
"""
import argparse
import sys
import time
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))
import splash_gb300 as sg  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mesh", default="hex", choices=["hex", "quad", "ico"])
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--solver", type=int, default=3, choices=[1, 2, 3])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--dt0", type=float, default=2e-4)
    ap.add_argument("--no-accretion", action="store_true")
    a = ap.parse_args()
    mesh = sg.Mesh({"hex": 0, "quad": 1, "ico": 2}[a.mesh], a.level)
    geom = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.quiet_noise(geom.unit_face_centers(), gam, seed=1)
    params = sg.SolverParams(accretion_rate=1e-2, e_acc=0.5, omega_acc_abs=0.5, tilt_angle=0.2,
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    prec = sg.PREC_MIXED if a.precision == "mixed" else sg.PREC_FP64
    s = sg.Solver(mesh, U0, 5, gam, 0.0, not a.no_accretion, params=params, solver=a.solver,
                  precision=prec)
    t0 = time.perf_counter()
    s.do_steps(a.steps, a.dt0)
    s.synchronize()
    dt = time.perf_counter() - t0
    print(f"{a.mesh}({a.level}) F={geom.n_faces} solver={a.solver} {a.precision}: "
          f"{a.steps} steps in {dt * 1e3:.2f} ms, stop={s.get_stop_check()}")


if __name__ == "__main__":
    main()
