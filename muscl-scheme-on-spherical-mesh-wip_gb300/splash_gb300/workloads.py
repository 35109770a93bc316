"""Seeded synthetic workloads shared by the benchmark and the tests.

The batched workload: many independent solvers on icosphere_hex meshes of
uneven size, each with its own accretion parameters and CFL dt.  There is
no dataset; every input is drawn from numpy's default_rng.
"""
from __future__ import annotations

import numpy as np

from . import initial_conditions as ic


def ensemble_draws(n_members: int = 512, seed: int = 3, levels=(3, 4, 5, 6, 7)) -> list[dict]:
    """Per-member choices of the batched workload, without building meshes.

    The mesh level is drawn with weights 2^-(level - min level) (small meshes
    favoured), dim 4 or 5 at 50/50.  Dim-5 members run MUSCL_HLLCplus with
    accretion_rate log-uniform in [1e-4, 1e-1], tilt_angle uniform in
    [0, pi/2], omega_acc_abs uniform in [0, 1], acc_width 0.1, e_acc 0.5,
    friction on, alpha 1e-6; dim-4 members run the isothermal MUSCL_HLLE
    (HLLC+ is adiabatic only; the isothermal solver has no source) and draw
    the same parameters, unused.  Member i's initial state is Sigma = Pi =
    1 +- 1e-3 from seed 1000 + i."""
    rng = np.random.default_rng(seed)
    levels = np.asarray(levels)
    w = 2.0 ** -(levels - levels.min())
    draw = rng.choice(levels, size=n_members, p=w / w.sum())
    dims = rng.choice([4, 5], size=n_members)
    out = []
    for i in range(n_members):
        p = {"accretion_rate": float(10 ** rng.uniform(-4, -1)), "e_acc": 0.5,
             "omega_acc_abs": float(rng.uniform(0, 1)), "tilt_angle": float(rng.uniform(0, np.pi / 2)),
             "acc_width": 0.1, "alpha": 1e-6, "friction_on": True}
        out.append({"index": i, "level": int(draw[i]), "dim": int(dims[i]), "params": p,
                    "ic_seed": 1000 + i})
    return out


def ensemble_members(sg, draws: list[dict], centres: dict | None = None) -> list[dict]:
    """Member dicts for splash_gb300.Ensemble from ensemble_draws() output.
    centres: optional cache {level: unit face centres}."""
    gam = ic.gam2d(4 / 3)
    centres = {} if centres is None else centres
    members = []
    for d in draws:
        lv = d["level"]
        if lv not in centres:
            centres[lv] = sg.Geometry(sg.icosphere_hex(lv)).unit_face_centers()
        U = ic.quiet_noise(centres[lv], gam, seed=d["ic_seed"])
        solver = sg.SOLVER_HLLCPLUS
        if d["dim"] == 4:
            solver, U = sg.SOLVER_HLLE, np.ascontiguousarray(U[:, :4])
        members.append({"mesh": sg.icosphere_hex(lv), "U_in": U, "gam": gam, "omega_ns": 0.0,
                        "accretion_on": True, "params": sg.SolverParams(**d["params"]),
                        "solver": solver})
    return members
