"""Benchmark of the GB300 MUSCL time step (one JSON line on rank 0).

Workload (the accreting mid-size configuration): icosphere_hex(7)
(163,842 faces), MUSCL_HLLCplus, dim 5, gam3d 4/3, omega_ns 0, accretion on
(rate 1e-2, e_acc 0.5, omega_acc 0.5, tilt 0.2, width 0.1, friction on,
alpha 1e-6), initial Sigma = Pi = 1 with 1e-3 uniform noise (seed 1), zero
velocity, dt0 = 2e-4.  Synthetic inputs; there is no dataset.

A "step" is one do_step(dt0): two RK stages over every face.  value is
face-updates/s (faces x steps / device time) with the state resident in
HBM; e2e is the same metric through the C ABI with host buffers (state
uploaded and read back every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
PKG = REPO / "muscl-scheme-on-spherical-mesh-wip_gb300"
for _p in (str(PKG), str(REPO)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "face-updates/s"
LEVEL = 7
DT0 = 2e-4
PARAMS = dict(accretion_rate=1e-2, e_acc=0.5, omega_acc_abs=0.5, tilt_angle=0.2, acc_width=0.1,
              alpha=1e-6, friction_on=True)


def measured_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, or None."""
    p = REPO / "profiles" / "traffic_hex7_mixed.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) == 2 and parts[0] == kernel and not line.startswith("#"):
            return float(parts[1])
    return None


def fp64_pipe_busy():
    """FP64-pipe utilisation of the FP64 path's kernels from the committed ncu
    summary (profiles/fp64_pipe_hex7.txt), or None."""
    p = REPO / "profiles" / "fp64_pipe_hex7.txt"
    if not p.exists():
        return None
    out = {}
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) == 2 and not line.startswith("#"):
            out[parts[0]] = float(parts[1])
    return {"per_kernel": out, "source": "profiles/fp64_pipe_hex7.txt (ncu sm__pipe_fp64_cycles_active)"} if out else None


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload_config(n_faces, precision_name):
    return {"workload": f"icosphere_hex({LEVEL}) MUSCL_HLLCplus dim5 accretion_on quiet-noise seed1",
            "n_faces": n_faces, "solver": "HLLCplus", "dt0": DT0, "precision": precision_name,
            "l2": "flushed: a 512 MB buffer is written on the solver stream before every timed step "
                  "(outside the CUDA-event intervals; the hex(7) mixed working set, working_set_mb in "
                  "decimal MB, is about the 129 MB L2); e2e flushed the same way between steps"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile(prefix="clocks_", suffix=".csv", delete=False)
        self.device = device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.tmp.close()

    def summary(self):
        rows = []
        try:
            for line in Path(self.tmp.name).read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------------ helpers
def build_case(sg):
    mesh = sg.icosphere_hex(LEVEL)
    geom = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    U0 = sg.initial_conditions.quiet_noise(geom.unit_face_centers(), gam, seed=1)
    return mesh, geom, gam, U0


L2_FLUSH_BYTES = 512 * 2**20  # written before every timed step (the L2 is 129 MB)


class L2Flush:
    """Writes a device buffer larger than the L2 on the solver's stream, so
    that the next step starts with no data of its own in the L2."""

    def __init__(self, torch, solver):
        self.stream = torch.cuda.ExternalStream(solver.stream())
        self.buf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        self.k = 0

    def __call__(self, torch):
        self.k = (self.k + 1) & 255
        with torch.cuda.stream(self.stream):
            self.buf.fill_(self.k)


def time_device_flushed(sg, torch, solver, n_faces, steps, warmup):
    """Device time of `steps` single steps on the solver's stream, the L2
    flushed before each (the flush outside the timed intervals): the sum of
    the per-step CUDA-event intervals."""
    stream = torch.cuda.ExternalStream(solver.stream())
    flush = L2Flush(torch, solver)
    for _ in range(warmup):
        flush(torch)
        solver.do_step(DT0)
    solver.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for a, b in ev:
        flush(torch)
        a.record(stream)
        solver.do_step(DT0)
        b.record(stream)
    ev[-1][1].synchronize()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3


def time_device(sg, torch, solver, n_faces, steps, warmup):
    """Device time of `steps` graph replays back to back on the solver's
    stream (no flush: for working sets larger than the L2)."""
    stream = torch.cuda.ExternalStream(solver.stream())
    for _ in range(warmup):
        solver.do_step(DT0)
    solver.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    solver.do_steps(steps, DT0)
    end.record(stream)
    end.synchronize()
    torch.cuda.synchronize()
    return start.elapsed_time(end) / 1e3


def pinned_like(torch, a):
    """A page-locked host array with a's shape and contents."""
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    out = t.numpy()
    out[...] = a
    return out


def time_e2e(sg, solver, U_host, steps, flush=None, torch=None):
    """Through the C ABI with host buffers, wall clock per step: the state
    uploaded from the host array (H2D), one do_step, the state read back
    (D2H), as one splash_do_steps_host call (one synchronisation per step).
    With `flush`, the L2 is flushed before every step outside the timed
    intervals."""
    out = np.empty_like(U_host) if torch is None else pinned_like(torch, np.zeros_like(U_host))
    solver.do_steps_host(U_host, 1, DT0, out)
    total = 0.0
    for _ in range(steps):
        if flush is not None:
            flush(torch)
            solver.synchronize()
        t0 = time.perf_counter()
        solver.do_steps_host(U_host, 1, DT0, out)
        total += time.perf_counter() - t0
    return total


def cpu_baseline(geom, U0, gam, budget_s=15.0):
    """The CPU oracle (restatement of the reference, OpenMP, all host cores)
    on a bounded sample of the same workload."""
    import splash_gb300 as sg
    from oracle.oracle import Oracle

    cores = os.cpu_count() or 1
    o = Oracle(geom, U0, gam, 0.0, True, sg.SolverParams(**PARAMS).as_list(), 3, threads=cores)
    o.do_step(DT0)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while n < 50:
        o.do_step(DT0)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    # one thread, a shorter sample of the same state
    o1 = Oracle(geom, U0, gam, 0.0, True, sg.SolverParams(**PARAMS).as_list(), 3, threads=1)
    t1 = time.perf_counter()
    n1 = 0
    while n1 < 10:
        o1.do_step(DT0)
        n1 += 1
        if time.perf_counter() - t1 > budget_s / 3:
            break
    dt1 = time.perf_counter() - t1
    return {"value": geom.n_faces * n / dt, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{n} do_step calls of the full workload after 1 warm-up "
                      f"({dt:.1f} s, OpenMP {cores} threads, {platform.machine()})",
            "value_1_thread": geom.n_faces * n1 / dt1, "sample_1_thread": f"{n1} do_step calls ({dt1:.1f} s)",
            "cpu_model": cpu_model()}


def cpu_model() -> str:
    """The host CPU's model name (or its architecture when none is listed)."""
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            key = line.split(":")[0].strip().lower()
            if key in ("model name", "cpu model", "hardware"):
                return line.split(":", 1)[1].strip()
        parts = [line.split(":", 1)[1].strip() for line in Path("/proc/cpuinfo").read_text().splitlines()
                 if line.lower().startswith(("cpu implementer", "cpu part"))][:2]
        if parts:
            return f"{platform.machine()} implementer {parts[0]} part {parts[1] if len(parts) > 1 else '?'}"
    except OSError:
        pass
    return platform.machine()


def step_bytes_mixed(geom) -> float:
    """Compulsory bytes of one mixed-precision step by the per-mesh formula
    bytes/step = 2 (b_slot S + b_edge E + b_face F) + 5 dim 8 F with the
    FP32-geometry sizes b_slot = 44 (4 stencil ids, 4 weights, H+, H-,
    BM_dist), b_edge = 36 (normal, centre, length, 2 face ids), b_face = 20
    (FP64 area, FP32 unit centre): the minimal data set, once per stage, and
    the five FP64 state accesses of a step."""
    F = geom.n_faces
    S = geom.n_slots
    E = S // 2
    return 2 * (44 * S + 36 * E + 20 * F) + 5 * 5 * 8 * F


def algorithmic_bytes_mixed(geom, kernel: str) -> float:
    """Compulsory bytes per launch of one kernel of the mixed path (F faces,
    S slots, E = S / 2 interior edges).

    edge (reconstruction + Riemann flux, one thread per edge): the edge
      record (face ids, edge centre, normal, n x R: 48 B) and per side the
      stencil, weights and distances (2 x 48 B); every face state read once
      (20 B per face); write the edge flux (20 B per edge).  (The stage-2
      edge states are no longer stored: the writers recompute them.)
    update (mean of the two stages): per face W32 (20 B), U0 (40 B), unit
      centre FP64 + FP32 (24 + 12 B), accretion source (8 B), slot count
      (1 B); per slot edge id and flux coefficient (8 B); every edge flux once
      (20 B per edge); write W32 (20 B) and, in stage 2, U (40 B).
    """
    F = geom.n_faces
    S = geom.n_slots
    E = S // 2
    if kernel == "edge":
        return E * (48 + 96 + 20) + F * 20
    return F * (20 + 40 + 24 + 12 + 8 + 1) + S * 8 + E * 20 + F * (20 + 40 / 2)


def algorithmic_bytes(geom, kernel: str) -> float:
    """Compulsory bytes per launch of one kernel of the FP64 path.

    reconstruct: read W (5 x 8 B per face), per slot 4 int32 stencil ids +
      4 betas + H+, H-, BM + edge centre (3) + |ec| + normal (3) + Courant
      factor + 2 eta (8 B each except ids) ; write U+ (5 x 8 B per slot).
    flux_update: read U+ (5 x 8 B per slot, each read once algorithmically),
      per slot edge centre, |ec|, normal, n x R, chord (11 x 8 B) + reverse
      index (4 B); per face W, U0, unit centre, area, accretion source
      (5+5+3+1+1 doubles) ; write U (or W1) and W (10 x 8 B).
    """
    F = geom.n_faces
    S = geom.n_slots
    if kernel == "reconstruct":
        return F * 40 + S * (16 + 8 * (4 + 3 + 3 + 1 + 3 + 1 + 2)) + S * 40
    return S * 40 + S * (11 * 8 + 4) + F * 8 * (5 + 5 + 3 + 1 + 1) + F * 80


# ------------------------------------------------------------------ arms
STOP_BITS = {1: "nan_flux", 2: "nan_wave_speed", 4: "wave_order", 8: "negative_extra_dt"}


def stop_bit_names(err: int) -> list[str]:
    """The stop causes in an error word (include/splash_gb300.h SPLASH_STOP_*)."""
    return [name for bit, name in STOP_BITS.items() if err & bit]


def ensemble_workload(sg, torch, steps=500, n_members=512, seed=3):
    """The batched workload: 512 independent members on icosphere_hex(3..7)
    (level drawn with weights 2^-(level-3), seed 3), mixed precision, dim 4
    or 5 drawn 50/50 (splash_gb300.workloads.ensemble_draws: dim-5 members
    run MUSCL_HLLCplus with their own accretion parameters, dim-4 members the
    isothermal MUSCL_HLLE).  Sigma = Pi = 1 +- 1e-3 (own seed); each member
    runs `steps` steps with its own CFL dt (dt0 = 1 never binds)."""
    from splash_gb300 import workloads

    draws = workloads.ensemble_draws(n_members, seed)
    draw = np.array([d["level"] for d in draws])
    dims = np.array([d["dim"] for d in draws])
    levels = np.arange(3, 8)
    members = workloads.ensemble_members(sg, draws)
    t0 = time.perf_counter()
    ens = sg.Ensemble(members, autotune=True)
    setup = time.perf_counter() - t0
    n, total = ens.size()
    stream = torch.cuda.ExternalStream(ens.stream())
    ens.do_steps(3, 1.0)
    ens.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ens.do_steps(steps, 1.0)
    b.record(stream)
    b.synchronize()
    secs = a.elapsed_time(b) / 1e3
    infos = [ens.member_info(i) for i in range(n)]
    sched = ens.schedule()
    # both designs timed over 100 more steps each: one persistent launch per
    # do_steps call, and five launches per step (the fastest width the
    # autotuner timed for the chosen tile order)
    order = ["member", "largest-first", "round-robin"].index(sched["order"])
    widths = [32, 64, 128]
    w5 = widths[int(np.argmin(sched["trial_ms"][order]))]
    designs = {}
    for name, width in (("persistent", 0), ("five_launches", w5)):
        try:
            ens.set_schedule(order, width)
        except sg.SplashError as exc:
            designs[name] = {"unavailable": str(exc)}
            continue
        ens.do_steps(2, 1.0)
        ens.synchronize()
        a.record(stream)
        ens.do_steps(100, 1.0)
        b.record(stream)
        b.synchronize()
        designs[name] = {"ms_per_step": a.elapsed_time(b) / 100, "edge_block": width}
    dts = [x["dt"] for x in infos]
    stops = sum(1 for x in infos if x["err"])
    # every member whose error word is non-zero, with what it latched
    stop_members = [{"member": i, "level": draws[i]["level"], "dim": draws[i]["dim"], "err": infos[i]["err"],
                     "bits": stop_bit_names(infos[i]["err"]), "params": draws[i]["params"]}
                    for i in range(n) if infos[i]["err"]]
    out = {"members": n, "total_faces": total, "levels_drawn": {int(l): int((draw == l).sum()) for l in levels},
           "steps": steps, "value": total * steps / secs, "unit": METRIC,
           "ms_per_step": secs / steps * 1e3, "setup_s": setup, "schedule": sched, "designs_100_steps": designs,
           "dt_range": [min(dts), max(dts)], "members_with_stop_flag": stops,
           "stop_members": stop_members,
           "dims_drawn": {"4": int((dims == 4).sum()), "5": int((dims == 5).sum())}}
    ens.close()
    return out


def adjoint_setup(sg, level=6, seed=4, solver=2, checkpoint_every=50):
    """The discrete-adjoint workload: icosphere_hex(level), MUSCL_HLLC (solver
    2), dim 5, FP64; rotating-blob initial state (seed 4); accretion on
    (e_acc 0.5, omega_acc_abs 0.5, width 0.1, friction on, alpha 1e-6);
    theta = (accretion_rate, tilt_angle, omega_acc_abs) = (1e-2, 0.1, 0.5)."""
    gam = sg.initial_conditions.gam2d(4 / 3)
    mesh = sg.icosphere_hex(level)
    geo = sg.Geometry(mesh)
    U0 = sg.initial_conditions.rotating_blob(geo.unit_face_centers(), gam, seed=seed)
    theta = np.array([1e-2, 0.1, 0.5])
    params = sg.SolverParams(accretion_rate=theta[0], e_acc=0.5, omega_acc_abs=theta[2], tilt_angle=theta[1],
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    base = sg.Solver(mesh, U0, 5, gam, 0.0, True, params=params, solver=solver, precision=sg.PREC_FP64)
    adj = sg.Adjoint(base, checkpoint_every=checkpoint_every)
    return base, adj, U0, theta, geo["area"].copy()


def fd_check(adj, U0, theta, gU, gth, target, area, steps, dt0, directions, h=1e-6):
    """Central differences of the loss 1/2 sum area (Sigma - Sigma*)^2 at
    step h along each direction (dU, dtheta), against the adjoint's
    directional derivative <gU, dU> + <gth, dtheta>.  The two runs at
    (U0, theta) +- h (dU, dtheta) are the plain FP64 forward compared with a
    branch recording made at (U0, theta) just before
    (splash_adjoint_branch_tape): `crossings` counts the (face, launch)
    evaluations whose branch path (limiter cases and min/max arguments,
    Riemann sides, floors) departs from the recorded one in either run,
    i.e. the kinks between the branches that the difference straddles and
    the adjoint, which differentiates the recorded branches, does not."""
    def loss(U):
        return 0.5 * math.fsum((area * (U[:, 0] - target) ** 2).tolist())

    rows = []
    for dU, dth in directions:
        g = float(np.sum(gU * dU) + np.dot(gth, dth))
        Up, cp = adj.branch_tape(U0 + h * dU, theta + h * dth, steps, "compare")
        Um, cm = adj.branch_tape(U0 - h * dU, theta - h * dth, steps, "compare")
        fd = (loss(Up) - loss(Um)) / (2 * h)
        rows.append({"adjoint": g, "plain_fd": fd, "rel": abs(fd - g) / abs(g), "crossings": cp + cm})
    return rows


def fd_summary(rows, evaluations):
    """Largest relative difference of a set of fd_check rows, and how many
    (face, launch) evaluations their runs departed at, of `evaluations` per
    run."""
    return {"n": len(rows), "max_rel": max((r["rel"] for r in rows), default=None),
            "max_crossings": max((r["crossings"] for r in rows), default=0),
            "evaluations_per_run": evaluations,
            "no_crossing_max_rel": max((r["rel"] for r in rows if r["crossings"] == 0), default=None)}


def adjoint_workload(sg, torch, steps=1000, checkpoint_every=50, level=6, seed=4, n_joint=16, n_param=5,
                     n_local=4, h=1e-6):
    """The discrete-adjoint workload (adjoint_setup), 1000 steps at dt0 =
    5e-4, checkpoints every 50 steps; loss 1/2 sum area (Sigma - Sigma*)^2
    against a run with accretion_rate 2e-2, tilt 0.3.  Cost = gradient time
    (forward with checkpoints + recomputing backward, CUDA events) over the
    plain FP64 forward of the same steps (graph replays, CUDA events).
    Derivative checks along seeded directions: the TLM (<lambda, J d> =
    <J^T lambda, d>), and central differences at h = 1e-6 of the forward
    itself and of the branch-frozen forward (fd_check), along n_joint
    joint directions (U0 with per-field scales of U0, and theta) and n_param
    parameter-only directions (the three unit ones first), and n_local
    state directions supported on the blob's core."""
    dt0 = 5e-4
    base, adj, U0, theta, area = adjoint_setup(sg, level, seed, 2, checkpoint_every)
    stream = torch.cuda.ExternalStream(base.stream())
    base.do_steps(3, dt0)
    base.synchronize()
    base.set_state(U0)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    base.do_steps(steps, dt0)
    b.record(stream)
    b.synchronize()
    fwd_ms = a.elapsed_time(b)
    target = adj.forward(U0, np.array([2e-2, 0.3, 0.5]), steps, dt0)[:, 0].copy()
    loss, gU, gth = adj.run(U0, theta, steps, dt0, target)
    info = adj.info()
    Uf = adj.forward(U0, theta, steps, dt0)
    rng = np.random.default_rng(seed)
    scale = np.maximum(np.abs(U0).max(axis=0), 1e-3)
    dU = rng.normal(size=U0.shape) * scale
    dth = rng.normal(size=3) * np.array([1e-2, 0.1, 0.5])
    _, dUt = adj.tlm(U0, theta, dU, dth, steps, dt0)
    tlm_ms = adj.info()["ms_tlm"]
    g_adj = float(np.sum(gU * dU) + np.dot(gth, dth))
    g_tlm = float(np.sum(area * (Uf[:, 0] - target) * dUt[:, 0]))
    # finite-difference checks: the seeded joint directions (the first is
    # the TLM's) and the parameter directions
    joint = [(dU, dth)] + [(rng.normal(size=U0.shape) * scale, rng.normal(size=3) * np.array([1e-2, 0.1, 0.5]))
                           for _ in range(n_joint - 1)]
    units = [np.array([1e-2, 0, 0]), np.array([0, 0.1, 0]), np.array([0, 0, 0.5])]
    params = (units + [rng.normal(size=3) * np.array([1e-2, 0.1, 0.5]) for _ in range(max(0, n_param - 3))])[:n_param]
    # state directions supported where the blob's density exceeds the far
    # field by more than 1e-2 (the far field is exactly uniform, and the
    # blob's tail is uniform to 1e-10, where a relative perturbation of h
    # decides the limiter ratios by itself)
    core = (U0[:, 0] - 1.0 > 1e-2).astype(float)[:, None]
    local = [(rng.normal(size=U0.shape) * scale * core, np.zeros(3)) for _ in range(n_local)]
    adj.forward(U0, theta, steps, dt0)  # the dt schedule the taped runs follow
    t0 = time.perf_counter()
    adj.branch_tape(U0, theta, steps, "record")
    tape_ms = (time.perf_counter() - t0) * 1e3  # wall clock, including the state upload
    evaluations = base.n_faces * (1 + 4 * steps)
    rows_j = fd_check(adj, U0, theta, gU, gth, target, area, steps, dt0, joint[:n_joint], h)
    pdirs = [(np.zeros_like(U0), d) for d in params]
    rows_p = fd_check(adj, U0, theta, gU, gth, target, area, steps, dt0, pdirs, h)
    rows_l = fd_check(adj, U0, theta, gU, gth, target, area, steps, dt0, local, h)
    # other steps straddle other kinks (the error follows the crossings, not
    # h^2: fourth-order differences do no better; it is not monotone in h),
    # until round-off sets in below about 3e-8
    sweep = {f"{hs:.0e}": {"parameter": fd_summary(fd_check(adj, U0, theta, gU, gth, target, area, steps, dt0,
                                                             pdirs, hs), evaluations),
                           "core_state": fd_summary(fd_check(adj, U0, theta, gU, gth, target, area, steps, dt0,
                                                              local, hs), evaluations)}
             for hs in (2e-7, 1e-7, 1e-8)}
    out = {"workload": f"icosphere_hex({level}) {base.n_faces} faces, HLLC, FP64, {steps} steps dt0={dt0}, "
                       f"checkpoints every {checkpoint_every}",
           "forward_ms": fwd_ms, "gradient_forward_ms": info["ms_forward"],
           "gradient_backward_ms": info["ms_backward"],
           "adjoint_over_forward": (info["ms_forward"] + info["ms_backward"]) / fwd_ms,
           "tlm_over_forward": tlm_ms / fwd_ms, "clipped_steps": info["clipped_steps"],
           "loss": loss, "grad_theta": gth.tolist(), "rel_adjoint_vs_tlm": abs(g_adj - g_tlm) / abs(g_tlm),
           "fd_h": h,
           "fd_parameter": fd_summary(rows_p, evaluations), "fd_core_state": fd_summary(rows_l, evaluations),
           "fd_joint": fd_summary(rows_j, evaluations),
           "fd_rows": {"joint": rows_j, "parameter": rows_p, "core_state": rows_l},
           "fd_smaller_h": sweep,
           "core_faces": int(core.sum()),
           "branch_tape_record_ms": tape_ms,
           "fd_note": "central differences of the FP64 forward at h; crossings: (face, launch) evaluations whose "
                      "branch path departs from the one at theta in the two runs, the kinks the difference "
                      "straddles (the adjoint differentiates the branches taken at theta)",
           "device_bytes": info["device_bytes"]}
    adj.close()
    base.close()
    return out


SHEAR_CASES = {
    # name: (mesh kind, level, solver, dim)
    "hex9_hllcp": (0, 9, 3, 5),   # icosphere_hex(9), 2,621,442 faces, MUSCL_HLLCplus
    "quad9_hllc": (1, 9, 2, 5),   # quad_sphere(9), 1,572,864 faces, MUSCL_HLLC
    "quad9_hlle": (1, 9, 4, 4),   # quad_sphere(9), isothermal MUSCL_HLLE (dim 4)
}


def timed_steps(torch, solver, steps, dt0):
    """CUDA-event time of `steps` do_step calls replayed back to back."""
    stream = torch.cuda.ExternalStream(solver.stream())
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    solver.do_steps(steps, dt0)
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / 1e3


def shear_workload(sg, torch, case="hex9_hllcp", steps=1000, seed=2, dt0=1e-4, warmup=3):
    """The large-mesh shear layer: u_phi = 0.5 tanh(latitude / 0.05), Sigma =
    1 + 1e-2 x random real Y_lm (l <= 8, seed 2), Pi = Sigma^gam2d, gam3d =
    4/3, no accretion, do_step(1e-4) with the CFL clip picking dt.  Both
    precisions run `steps` steps from the same state (state resident; the
    working sets are GBs, far larger than the L2).  Reported: face-updates/s
    of each, mixed/FP64, the mixed state's relative L1 and L-infinity error
    per field against FP64 (angular momentum also against the momentum scale
    Sigma c_s), total mass and angular-momentum drift of each run, the last
    dt and the stop flags."""
    kind, level, solver_kind, dim = SHEAR_CASES[case]
    mesh = sg.Mesh(kind, level)
    gam = sg.initial_conditions.gam2d(4 / 3)
    t0 = time.perf_counter()
    geo = sg.Geometry(mesh)
    r, area = geo.unit_face_centers(), geo["area"].copy()
    nf = geo.n_faces
    del geo
    U0 = np.ascontiguousarray(sg.initial_conditions.shear_layer(r, gam, seed=seed)[:, :dim])
    setup = {"geometry_s": time.perf_counter() - t0}
    out = {"workload": f"{['icosphere_hex', 'quad_sphere'][kind]}({level}) {nf} faces, solver {solver_kind}, "
                       f"dim {dim}, shear layer seed {seed}, dt0={dt0} (CFL-clipped)",
           "faces": nf, "steps": steps, "unit": METRIC}
    states = {}
    for name, prec in (("fp64", sg.PREC_FP64), ("mixed", sg.PREC_MIXED)):
        t0 = time.perf_counter()
        s = sg.Solver(mesh, U0, dim, gam, 0.0, False, params=sg.SolverParams(), solver=solver_kind,
                      precision=prec)
        setup[f"create_{name}_s"] = time.perf_counter() - t0
        s.do_steps(warmup, dt0)
        s.synchronize()
        s.set_state(U0)
        d0 = s.diagnostics()
        secs = timed_steps(torch, s, steps, dt0)
        d1 = s.diagnostics()
        states[name] = s.get_state()
        out[name] = {"value": nf * steps / secs, "ms_per_step": secs / steps * 1e3, "t": s.time(),
                     "last_dt": s.last_dt(), "stop": s.get_stop_check(), "error_word": s.error_word(),
                     "mass_drift": float(d1[0] / d0[0] - 1),
                     "angular_momentum_drift": drift_l(d0, d1, U0, area)}
        s.close()
    a, b = states["fp64"], states["mixed"]
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["l1_rel_per_field"] = l1_rel(b, a, area).tolist()
    out["linf_rel_per_field"] = (np.max(np.abs(b - a), axis=0) /
                                 np.maximum(np.max(np.abs(a), axis=0), 1e-300)).tolist()
    out["l1_angular_momentum_vs_sigma_cs"] = l1_momentum_scale(b, a, area, gam, dim).tolist()
    out["setup_s"] = setup
    return out


def drift_l(d0, d1, U0, area) -> float:
    """|L(t) - L(0)| over the total absolute angular momentum sum A |l| of the
    initial state (the total L of a symmetric flow can be ~0)."""
    scale = float(np.sum(area * np.linalg.norm(U0[:, 1:4], axis=1)))
    return float(np.linalg.norm(np.asarray(d1[1:4]) - np.asarray(d0[1:4])) / max(scale, 1e-300))


def l1_momentum_scale(a, b, area, gam, dim=5):
    """Relative L1 of the angular-momentum fields against the momentum scale
    Sigma c_s (c_s the sound speed of b; the isothermal c_s is 1):
    sum A |l_a - l_b| / sum A Sigma_b c_s."""
    if dim == 5:
        cs = np.sqrt(np.maximum(gam * pressure_of(b, gam) / b[:, 0], 0.0))
    else:
        cs = np.ones(len(b))
    den = np.sum(area * b[:, 0] * cs)
    return np.sum(area[:, None] * np.abs(a[:, 1:4] - b[:, 1:4]), axis=0) / den


def pressure_of(U, gam):
    """Pi = (E - |l|^2 / (2 Sigma)) (gam - 1): |v| = |r x l| / Sigma = |l| / Sigma
    for tangential l (MUSCL_base.hpp:517-539, without the 1e-16 floor)."""
    l2 = np.sum(U[:, 1:4] * U[:, 1:4], axis=1)
    return (U[:, 4] - l2 / (2 * U[:, 0])) * (gam - 1)


def l1_rel(a, b, area):
    num = np.sum(area[:, None] * np.abs(a - b), axis=0)
    den = np.sum(area[:, None] * np.abs(b), axis=0)
    return num / np.where(den > 0, den, 1)


def max_over_ranks(torch, secs: float, world: int, device: str) -> float:
    """The largest timed-region length over all ranks (every rank runs one
    full replica; the whole job ends when the slowest does).  device: where
    the reduction tensor lives ("cuda" for NCCL, "cpu" for gloo)."""
    if world <= 1:
        return secs
    t = torch.tensor([secs], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: int, steps: int, world: int, secs_max: float) -> float:
    """Whole-job throughput: the units every rank processed, over the
    slowest rank's time (weak scaling: each rank's work is fixed)."""
    return units_per_rank * steps * world / secs_max


def run_ours(args):
    import torch

    import splash_gb300 as sg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    mesh, geom, gam, U0 = build_case(sg)
    params = sg.SolverParams(**PARAMS)
    F = geom.n_faces
    mixed = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, True, params=params, precision=sg.PREC_MIXED,
                              device=local)
    fp64 = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, True, params=params, precision=sg.PREC_FP64,
                             device=local)
    dm0, d640 = mixed.diagnostics(), fp64.diagnostics()
    # one full replica per GPU: the step does not shard
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        # the hex(7) mixed working set is about the L2 size: flush before each step
        secs = time_device_flushed(sg, torch, mixed, F, args.steps, args.warmup)
        secs = max_over_ranks(torch, secs, world, "cuda")
    clk = clocks.summary()
    value = job_value(F, args.steps, world, secs)
    secs64 = time_device(sg, torch, fp64, F, args.steps, args.warmup)
    value64 = F * args.steps / secs64
    # accuracy of the timed runs: both advanced warmup + steps from the same state
    Um, U64 = mixed.get_state(), fp64.get_state()
    area = geom["area"]
    dm1, d641 = mixed.diagnostics(), fp64.diagnostics()
    acc = {"steps": args.warmup + args.steps, "l1_rel_per_field": l1_rel(Um, U64, area).tolist(),
           "linf_rel_per_field": (np.max(np.abs(Um - U64), axis=0) /
                                  np.max(np.abs(U64), axis=0)).tolist(),
           # l starts at ~0 (the flow starts at rest), so its error is also
           # measured against the momentum scale Sigma c_s
           "l1_angular_momentum_vs_sigma_cs": l1_momentum_scale(Um, U64, area, gam).tolist(),
           "mass_change": {"mixed": float(dm1[0] / dm0[0] - 1), "fp64": float(d641[0] / d640[0] - 1),
                           "note": "relative change of the total mass over the run (accretion adds mass)"},
           "mass_mixed_vs_fp64": float(dm1[0] / d641[0] - 1),
           "angular_momentum_mixed_vs_fp64": float(np.linalg.norm(dm1[1:4] - d641[1:4]) /
                                                   np.sum(area * U64[:, 0] * np.sqrt(
                                                       gam * pressure_of(U64, gam) / U64[:, 0]))),
           "reference": "GPU FP64 path (1e-10 of the reference on the golden states)"}
    # per-kernel device times (un-captured launches, CUDA events on the solver stream)
    reps = max(3, min(20, args.steps))
    lt = mixed.launch_times(reps, DT0)
    ms64 = fp64.kernel_times(reps, DT0)
    # mean ms per launch of each kernel, and each kernel's ms per step
    # (slots: dt clip (empty: the stage-1 edge launch clips dt), edge 1, update 1, edge 2, update 2)
    kern = {"dt_clip_slot": lt[0], "edge": (lt[1] + lt[3]) / 2, "update": (lt[2] + lt[4]) / 2,
            "edge_stage1": lt[1], "edge_stage2": lt[3], "update_stage1": lt[2], "update_stage2": lt[4]}
    per_step = {"edge": lt[1] + lt[3], "update": lt[2] + lt[4]}
    kern64 = {"dt_reduce": ms64[0], "reconstruct": (ms64[1] + ms64[3]) / 2,
              "flux_update": (ms64[2] + ms64[4]) / 2}
    dom = max(per_step, key=per_step.get)
    hbm, src = peaks()
    ach = algorithmic_bytes_mixed(geom, dom) / (kern[dom] * 1e-3) / 1e9
    geo_b, st_b = mixed.memory()
    # end to end through the C ABI with host buffers
    U_host = pinned_like(torch, mixed.get_state())
    e2e_steps = max(3, min(args.steps, 50))
    e2e_secs = time_e2e(sg, mixed, U_host, e2e_steps, flush=L2Flush(torch, mixed), torch=torch)
    # the same step back to back in 4-step graphs, without flushes (steady
    # state of a run; the L2 then holds part of the working set)
    secs_bb = time_device(sg, torch, mixed, F, args.steps, args.warmup)
    bytes_io = F * 5 * 8
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {**workload_config(F, "mixed FP32/FP64"), "parallelism": f"replicas{world}",
                   "working_set_mb": round((geo_b + st_b) / 1e6, 1)},
        "gpu_launches": 4 * args.steps,
        "e2e": {"value": F * e2e_steps / e2e_secs, "unit": METRIC, "h2d_bytes_per_step": bytes_io,
                "d2h_bytes_per_step": bytes_io, "host_buffers": "pinned (page-locked) FP64 [F][5] arrays",
                "call": "splash_do_steps_host(s, U_in, 1, dt0, U_out) per step"},
        "fp64": {"value": value64, "ms_per_step": secs64 / args.steps * 1e3, "kernel_ms": kern64,
                 "fp64_pipe_busy": fp64_pipe_busy()},
        "back_to_back": {"value": F * args.steps / secs_bb, "ms_per_step": secs_bb / args.steps * 1e3,
                         "note": "do_steps in 4-step graphs, no L2 flush"},
        "mixed_over_fp64": value / value64,
        "accuracy": acc,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm,
                     "unit": "GB/s", "frac": ach / hbm, "traffic": measured_traffic(dom),
                     "algorithmic_bytes": algorithmic_bytes_mixed(geom, dom),
                     "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel_ms": kern, "kernel_ms_per_step": per_step},
        "roofline_step": {"bound": "hbm", "bytes_per_step": step_bytes_mixed(geom),
                          "bytes_per_face_update": step_bytes_mixed(geom) / F,
                          "achieved": step_bytes_mixed(geom) / (secs / args.steps) / 1e9, "peak": hbm,
                          "unit": "GB/s", "frac": step_bytes_mixed(geom) / (secs / args.steps) / 1e9 / hbm},
        "clocks": clk,
    }
    mixed.close()
    fp64.close()
    if not args.no_ensemble:
        line["ensemble"] = ensemble_workload(sg, torch)
    if not args.no_adjoint:
        line["adjoint"] = adjoint_workload(sg, torch, n_joint=args.adjoint_joint, n_param=args.adjoint_param,
                                           n_local=args.adjoint_local)
    if not args.no_shear:
        for i, case in enumerate(args.shear_cases):
            line["shear_layer" if i == 0 else f"shear_layer_{case}"] = shear_workload(
                sg, torch, case, steps=args.shear_steps)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(geom, U0, gam)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    """The reference's CPU path on the host cores: the reference itself cannot
    travel to the GPU host (its x86 build is not portable and its sources are
    not shipped), so its restatement in oracle/ (bit-identical to the
    reference on x86-64) runs with all host threads on the same workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import splash_gb300 as sg

    mesh, geom, gam, U0 = build_case(sg)
    from oracle.oracle import Oracle

    cores = os.cpu_count() or 1
    o = Oracle(geom, U0, gam, 0.0, True, sg.SolverParams(**PARAMS).as_list(), 3, threads=cores)
    # the same warm-up (at least 3) and step counts as the GPU arm: a hex(7)
    # oracle step takes tens of ms on the host cores
    warm = max(3, args.warmup)
    for _ in range(warm):
        o.do_step(DT0)
    n = max(1, args.steps)
    t0 = time.perf_counter()
    o.do_steps(n, DT0)
    secs = time.perf_counter() - t0
    value = geom.n_faces * n / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0,
        "steps": n, "warmup": warm, "ms_per_step": secs / n * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(geom.n_faces, "fp64"),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{n} do_step calls of the full workload, OpenMP {cores} "
                                   f"threads ({platform.machine()})"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile(args):
    """A profiler harness: builds one solver (or the adjoint) and runs a few
    steps, nothing else, so that an ncu capture sees only the step's kernels.

    --profile mixed|fp64: `--profile-steps` do_step replays of the given mesh
      and solver; initial state Sigma = Pi = 1 +- 1e-3 (seed 1), accretion on
      with the mid-size workload's parameters.
    --profile adjoint: one gradient (checkpointed forward + backward) of the
      adjoint workload at reduced length (rotating blob, seed 4; HLLC; dt0 =
      5e-4; loss target from accretion_rate 2e-2, tilt 0.3), then with --tlm
      one tangent-linear run."""
    import splash_gb300 as sg

    mesh = sg.Mesh({"hex": 0, "quad": 1, "ico": 2}[args.mesh], args.level)
    geom = sg.Geometry(mesh)
    gam = sg.initial_conditions.gam2d(4 / 3)
    if args.profile == "adjoint":
        U0 = sg.initial_conditions.rotating_blob(geom.unit_face_centers(), gam, seed=4)
        theta = np.array([1e-2, 0.1, 0.5])
        params = sg.SolverParams(accretion_rate=theta[0], e_acc=0.5, omega_acc_abs=theta[2],
                                 tilt_angle=theta[1], acc_width=0.1, alpha=1e-6, friction_on=True)
        base = sg.Solver(mesh, U0, 5, gam, 0.0, True, params=params, solver=args.solver,
                         precision=sg.PREC_FP64)
        adj = sg.Adjoint(base, checkpoint_every=args.checkpoint_every)
        target = adj.forward(U0, np.array([2e-2, 0.3, 0.5]), args.profile_steps, 5e-4)[:, 0].copy()
        loss, _, gth = adj.run(U0, theta, args.profile_steps, 5e-4, target)
        info = adj.info()
        print(f"{args.mesh}({args.level}) F={base.n_faces} solver={args.solver}: {args.profile_steps} steps, "
              f"K={args.checkpoint_every}: forward {info['ms_forward']:.2f} ms, backward "
              f"{info['ms_backward']:.2f} ms, loss {loss:.6e}, grad_theta {gth}")
        if args.tlm:
            rng = np.random.default_rng(0)
            adj.tlm(U0, theta, rng.normal(size=U0.shape), None, args.profile_steps, 5e-4)
            print(f"tlm {adj.info()['ms_tlm']:.2f} ms")
        adj.close()
        base.close()
        return
    U0 = sg.initial_conditions.quiet_noise(geom.unit_face_centers(), gam, seed=1)
    prec = sg.PREC_MIXED if args.profile == "mixed" else sg.PREC_FP64
    s = sg.Solver(mesh, U0, 5, gam, 0.0, True, params=sg.SolverParams(**PARAMS), solver=args.solver,
                  precision=prec)
    t0 = time.perf_counter()
    s.do_steps(args.profile_steps, DT0)
    s.synchronize()
    dt = time.perf_counter() - t0
    print(f"{args.mesh}({args.level}) F={geom.n_faces} solver={args.solver} {args.profile}: "
          f"{args.profile_steps} steps in {dt * 1e3:.2f} ms, stop={s.get_stop_check()}")
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-shear", action="store_true")
    ap.add_argument("--shear-cases", nargs="*", default=["hex9_hllcp"], choices=list(SHEAR_CASES),
                    help="large-mesh shear-layer cases, 1000 steps each in both precisions")
    ap.add_argument("--shear-steps", type=int, default=1000)
    ap.add_argument("--adjoint-joint", type=int, default=4,
                    help="joint (state + parameter) directions of the adjoint's finite-difference check")
    ap.add_argument("--adjoint-param", type=int, default=3, help="parameter-only directions of that check")
    ap.add_argument("--adjoint-local", type=int, default=2,
                    help="state directions supported on the blob's core, of that check")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the adjoint workload and print its JSON object (the full check: "
                         "--adjoint-joint 16 --adjoint-param 8)")
    # profiler harness (no JSON line): see run_profile
    ap.add_argument("--profile", choices=["mixed", "fp64", "adjoint"], default=None)
    ap.add_argument("--mesh", default="hex", choices=["hex", "quad", "ico"])
    ap.add_argument("--level", type=int, default=LEVEL)
    ap.add_argument("--solver", type=int, default=3, choices=[1, 2, 3])
    ap.add_argument("--profile-steps", type=int, default=5)
    ap.add_argument("--checkpoint-every", type=int, default=10)
    ap.add_argument("--tlm", action="store_true")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.adjoint_only:
        import torch

        import splash_gb300 as sg

        print(json.dumps(adjoint_workload(sg, torch, n_joint=args.adjoint_joint, n_param=args.adjoint_param,
                                          n_local=args.adjoint_local)), flush=True)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
