"""Shared test helpers: fixture loading, oracle construction, error norms."""
from __future__ import annotations

import platform
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
MESH_KIND = {"hex": 0, "quad": 1, "ico": 2}
# x86-64 runs both the reference and the restatements with the same libm and
# without FMA, so bit-exactness is expected there.
BIT_EXACT_HOST = platform.machine() in ("x86_64", "AMD64")


def load(name: str) -> dict:
    with np.load(GOLDEN / name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def mesh_of(kind: str, level: int):
    import splash_gb300 as sg

    return sg.Mesh(MESH_KIND[str(kind)], int(level))


def rel_linf(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per conserved field: max |a - b| / max |b| (a column per field)."""
    a = np.asarray(a).reshape(-1, a.shape[-1])
    b = np.asarray(b).reshape(-1, b.shape[-1])
    scale = np.max(np.abs(b), axis=0)
    scale = np.where(scale > 0, scale, 1.0)
    return np.max(np.abs(a - b), axis=0) / scale


def make_oracle(geom, case: dict, threads: int = 0, dim: int = 5):
    from oracle.oracle import Oracle

    return Oracle(geom, case["U0"], float(case["gam"]), 0.0, bool(case["accretion_on"]),
                  [float(x) for x in case["params"]], int(case["solver"]), threads=threads, dim=dim)
