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
    """Through the C ABI with host buffers: set_state (H2D), do_step,
    get_state (D2H) per step, wall clock.  With `flush`, the L2 is flushed
    before every step outside the timed intervals."""
    out = np.empty_like(U_host) if torch is None else pinned_like(torch, np.zeros_like(U_host))
    solver.set_state(U_host)
    solver.do_step(DT0)
    solver.get_state(out)
    total = 0.0
    for _ in range(steps):
        if flush is not None:
            flush(torch)
            solver.synchronize()
        t0 = time.perf_counter()
        solver.set_state(U_host)
        solver.do_step(DT0)
        solver.get_state(out)
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
      stencil, weights and distances (2 x 48 B); every face
      state W32 read once (20 B per face); write the edge flux (20 B per
      edge) and, in stage 2, both edge states (2 x 20 B per edge; mean of the
      two stages).
    update (mean of the two stages): per face W32 (20 B), U0 (40 B), unit
      centre FP64 + FP32 (24 + 12 B), accretion source (8 B), slot count
      (1 B); per slot edge id and flux coefficient (8 B); every edge flux once
      (20 B per edge); write W32 (20 B) and, in stage 2, U (40 B).
    """
    F = geom.n_faces
    S = geom.n_slots
    E = S // 2
    if kernel == "edge":
        return E * (48 + 96 + 20 + 40 / 2) + F * 20
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
def ensemble_workload(sg, torch, steps=500, n_members=512, seed=3):
    """The batched workload: 512 independent members on icosphere_hex(3..7)
    (level drawn with weights 2^-(level-3), seed 3), mixed precision, dim 4
    or 5 drawn 50/50: dim 5 members run MUSCL_HLLCplus with per-member
    accretion_rate log-uniform in [1e-4, 1e-1], tilt_angle uniform in
    [0, pi/2], omega_acc_abs uniform in [0, 1], acc_width 0.1, e_acc 0.5;
    dim 4 members run the isothermal MUSCL_HLLE (HLLC+ is adiabatic only, and
    the isothermal solver has no source).  Sigma = Pi = 1 +- 1e-3 (own seed);
    each member runs `steps` steps with its own CFL dt (dt0 = 1 never
    binds)."""
    rng = np.random.default_rng(seed)
    levels = np.arange(3, 8)
    w = 2.0 ** -(levels - 3)
    draw = rng.choice(levels, size=n_members, p=w / w.sum())
    dims = rng.choice([4, 5], size=n_members)
    gam = sg.initial_conditions.gam2d(4 / 3)
    centres = {}
    members = []
    for i, lv in enumerate(draw):
        lv = int(lv)
        if lv not in centres:
            centres[lv] = sg.Geometry(sg.icosphere_hex(lv)).unit_face_centers()
        U = sg.initial_conditions.quiet_noise(centres[lv], gam, seed=1000 + i)
        params = sg.SolverParams(accretion_rate=float(10 ** rng.uniform(-4, -1)), e_acc=0.5,
                                 omega_acc_abs=float(rng.uniform(0, 1)),
                                 tilt_angle=float(rng.uniform(0, np.pi / 2)), acc_width=0.1,
                                 alpha=1e-6, friction_on=True)
        solver = sg.SOLVER_HLLCPLUS
        if dims[i] == 4:
            solver, U = sg.SOLVER_HLLE, np.ascontiguousarray(U[:, :4])
        members.append({"mesh": sg.icosphere_hex(lv), "U_in": U, "gam": gam, "omega_ns": 0.0,
                        "accretion_on": True, "params": params, "solver": solver})
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
    dts = [ens.member_info(i)["dt"] for i in range(n)]
    stops = sum(1 for i in range(n) if ens.member_info(i)["err"])
    out = {"members": n, "total_faces": total, "levels_drawn": {int(l): int((draw == l).sum()) for l in levels},
           "steps": steps, "value": total * steps / secs, "unit": METRIC,
           "ms_per_step": secs / steps * 1e3, "setup_s": setup, "schedule": ens.schedule(),
           "dt_range": [min(dts), max(dts)], "members_with_stop_flag": stops,
           "dims_drawn": {"4": int((dims == 4).sum()), "5": int((dims == 5).sum())}}
    ens.close()
    return out


def adjoint_workload(sg, torch, steps=1000, checkpoint_every=50, level=6, seed=4):
    """The discrete-adjoint workload: icosphere_hex(6), HLLC, dim 5, FP64,
    1000 steps at dt0 = 5e-4, checkpoints every 50 steps; rotating-blob
    initial state (seed 4); accretion on (rate 1e-2, tilt 0.1, omega_acc 0.5,
    width 0.1, e_acc 0.5, friction on); loss 1/2 sum area (Sigma - Sigma*)^2
    against a run with rate 2e-2, tilt 0.3.  Cost = gradient time (forward
    with checkpoints + recomputing backward, CUDA events) over the plain FP64
    forward of the same steps (graph replays, CUDA events); one seeded
    direction is checked against the tangent-linear model."""
    dt0 = 5e-4
    gam = sg.initial_conditions.gam2d(4 / 3)
    mesh = sg.icosphere_hex(level)
    geo = sg.Geometry(mesh)
    U0 = sg.initial_conditions.rotating_blob(geo.unit_face_centers(), gam, seed=seed)
    theta = np.array([1e-2, 0.1, 0.5])
    params = sg.SolverParams(accretion_rate=theta[0], e_acc=0.5, omega_acc_abs=theta[2], tilt_angle=theta[1],
                             acc_width=0.1, alpha=1e-6, friction_on=True)
    base = sg.MUSCL_HLLC(mesh, U0, 5, gam, 0.0, True, params=params, precision=sg.PREC_FP64)
    adj = sg.Adjoint(base, checkpoint_every=checkpoint_every)
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
    dU = rng.normal(size=U0.shape) * np.maximum(np.abs(U0).max(axis=0), 1e-3)
    dth = rng.normal(size=3) * np.array([1e-2, 0.1, 0.5])
    _, dUt = adj.tlm(U0, theta, dU, dth, steps, dt0)
    tlm_ms = adj.info()["ms_tlm"]
    g_adj = float(np.sum(gU * dU) + np.dot(gth, dth))
    g_tlm = float(np.sum(geo["area"] * (Uf[:, 0] - target) * dUt[:, 0]))
    out = {"workload": f"icosphere_hex({level}) {base.n_faces} faces, HLLC, FP64, {steps} steps dt0={dt0}, "
                       f"checkpoints every {checkpoint_every}",
           "forward_ms": fwd_ms, "gradient_forward_ms": info["ms_forward"],
           "gradient_backward_ms": info["ms_backward"],
           "adjoint_over_forward": (info["ms_forward"] + info["ms_backward"]) / fwd_ms,
           "tlm_over_forward": tlm_ms / fwd_ms, "clipped_steps": info["clipped_steps"],
           "loss": loss, "grad_theta": gth.tolist(), "rel_adjoint_vs_tlm": abs(g_adj - g_tlm) / abs(g_tlm),
           "device_bytes": info["device_bytes"]}
    adj.close()
    base.close()
    return out


def shear_workload(sg, torch, fp64_steps=20, mixed_steps=200, level=9, seed=2, dt0=1e-4):
    """The large-mesh shear layer at reduced length: icosphere_hex(9)
    (2,621,442 faces), MUSCL_HLLCplus, dim 5, no accretion, u_phi = 0.5
    tanh(latitude / 0.05), Sigma = 1 + 1e-2 random Y_lm (l <= 8, seed 2),
    Pi = Sigma^gam2d, do_step(1e-4) with the CFL clip.  Both precisions run
    `fp64_steps` steps from the same state (face-updates/s of each and the
    mixed state's error against FP64 after those steps); the mixed path then
    runs `mixed_steps` more for its rate.  The 1000-step comparison of the
    full workload is shear_check.py."""
    gam = sg.initial_conditions.gam2d(4 / 3)
    mesh = sg.icosphere_hex(level)
    nf = 10 * 4 ** level + 2
    t0 = time.perf_counter()
    fp64 = sg.MUSCL_HLLCplus(mesh, np.ones((nf, 5)), 5, gam, 0.0, False, precision=sg.PREC_FP64)
    r, area = fp64.face_geometry()
    U0 = sg.initial_conditions.shear_layer(r, gam, seed=seed)
    mixed = sg.MUSCL_HLLCplus(mesh, U0, 5, gam, 0.0, False, precision=sg.PREC_MIXED)
    setup = time.perf_counter() - t0

    def timed(s, n):
        stream = torch.cuda.ExternalStream(s.stream())
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s.do_steps(n, dt0)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3

    for s in (fp64, mixed):
        s.do_steps(3, dt0)
        s.synchronize()
        s.set_state(U0)
    t64 = timed(fp64, fp64_steps)
    t32 = timed(mixed, fp64_steps)
    U64, U32 = fp64.get_state(), mixed.get_state()
    t32b = timed(mixed, mixed_steps)
    out = {"workload": f"icosphere_hex({level}) {nf} faces, HLLC+, shear layer, dt0={dt0} (CFL-clipped)",
           "fp64": {"value": nf * fp64_steps / t64, "ms_per_step": t64 / fp64_steps * 1e3, "steps": fp64_steps},
           "mixed": {"value": nf * mixed_steps / t32b, "ms_per_step": t32b / mixed_steps * 1e3,
                     "steps": mixed_steps},
           "unit": METRIC, "mixed_over_fp64": (nf * mixed_steps / t32b) / (nf * fp64_steps / t64),
           "l1_rel_per_field_after_fp64_steps": l1_rel(U32, U64, area).tolist(),
           "last_dt": fp64.last_dt(), "setup_s": setup}
    fp64.close()
    mixed.close()
    return out


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
    acc = {"steps": args.warmup + args.steps, "l1_rel_per_field": l1_rel(Um, U64, geom["area"]).tolist(),
           "linf_rel_per_field": (np.max(np.abs(Um - U64), axis=0) /
                                  np.max(np.abs(U64), axis=0)).tolist(),
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
                "d2h_bytes_per_step": bytes_io, "host_buffers": "pinned (page-locked) FP64 [F][5] arrays"},
        "fp64": {"value": value64, "ms_per_step": secs64 / args.steps * 1e3, "kernel_ms": kern64},
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
        line["adjoint"] = adjoint_workload(sg, torch)
    if not args.no_shear:
        line["shear_layer"] = shear_workload(sg, torch)
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
    # at least 3 warm-up steps like the GPU arm (a hex(7) oracle step takes
    # tens of ms on the host cores), at most 10; a bounded sample of at most
    # 10 timed steps
    warm = max(3, min(args.warmup, 10))
    for _ in range(warm):
        o.do_step(DT0)
    n = max(1, min(args.steps, 10))
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
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
