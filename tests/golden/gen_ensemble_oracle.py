"""Runs every member of the 512-member batched workload on the CPU oracle and
writes tests/golden/ensemble_oracle_c3.json.

The workload is splash_gb300.workloads.ensemble_draws(512, 3): icosphere_hex
(3..7) meshes, dims 4 and 5, per-member accretion parameters, Sigma = Pi =
1 +- 1e-3.  Each member runs 503 do_step(1.0) calls (3 warm-up + 500 timed
steps of the benchmark; dt0 = 1 never binds, the CFL clip picks every dt)
on the oracle (FP64, the reference restated and pinned bit-for-bit to it on
x86-64).  Per member the record keeps: the stop bits raised over the run,
the step at which each bit was first raised, the final time, the last dt,
and the total mass and energy sum area * (Sigma, E).

Usage:  python tests/golden/gen_ensemble_oracle.py [--procs 8]
About 25 minutes on 8 x86 cores (one oracle thread per member); it is never
run by the test-suite (the record is committed).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
STEPS = 503


def _paths():
    for p in (str(REPO / "muscl-scheme-on-spherical-mesh-wip_gb300"), str(REPO)):
        if p not in sys.path:
            sys.path.insert(0, p)


def run_member(d: dict) -> dict:
    _paths()
    import numpy as np

    import splash_gb300 as sg
    from oracle.oracle import Oracle
    from splash_gb300 import workloads

    geo = sg.Geometry(sg.icosphere_hex(d["level"]), threads=1)
    m = workloads.ensemble_members(sg, [d], {d["level"]: geo.unit_face_centers()})[0]
    o = Oracle(geo, m["U_in"], m["gam"], 0.0, True, m["params"].as_list(), m["solver"], threads=1, dim=d["dim"])
    bits, first = 0, {}
    for k in range(STEPS):
        b = o.do_step(1.0)
        for bit in (1, 2, 4, 8):
            if b & bit and str(bit) not in first:
                first[str(bit)] = k + 1
        bits |= b
    info = o.info()
    U = o.get_state()
    area = np.asarray(geo["area"])
    out = {"index": d["index"], "level": d["level"], "dim": d["dim"], "bits": bits, "first_step": first,
           "t": info["t"], "dt": info["dt"], "mass": float(np.sum(area * U[:, 0]))}
    if d["dim"] == 5:
        out["energy"] = float(np.sum(area * U[:, 4]))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=8)
    a = ap.parse_args()
    _paths()
    from splash_gb300 import workloads

    draws = sorted(workloads.ensemble_draws(512, 3), key=lambda d: -d["level"])  # large meshes first
    t0 = time.time()
    res = []
    with mp.get_context("spawn").Pool(a.procs) as pool:
        for r in pool.imap_unordered(run_member, draws):
            res.append(r)
    res.sort(key=lambda r: r["index"])
    rec = {"workload": "splash_gb300.workloads.ensemble_draws(512, 3)", "steps": STEPS, "dt0": 1.0,
           "members": res}
    (HERE / "ensemble_oracle_c3.json").write_text(json.dumps(rec, indent=0))
    stops = [(r["index"], r["level"], r["dim"], r["bits"], r["first_step"]) for r in res if r["bits"]]
    print(f"{len(res)} members in {time.time() - t0:.0f} s; members with stop bits: {stops}")


if __name__ == "__main__":
    main()
