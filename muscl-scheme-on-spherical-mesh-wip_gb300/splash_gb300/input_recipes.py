"""The reference's initial-condition recipes (make_input.py), without pandas.

Each recipe takes the unit face centres as the solver writes them to
results/face_centers.dat (``read_face_centers``; the C++ writer prints 15
significant digits, so the recipes see rounded centres, as in the
reference's workflow) and returns the conserved state U [F, dim] that the
reference would write to input/input.dat, with the text format its pandas
writer uses (``write_input_dat``).  The arithmetic follows the reference
expression by expression (numpy ufuncs in the same order, per-row vector
norms through the same dot product), so the arrays are bit-identical to
what the reference computes on the same face centres.

    python -m splash_gb300.input_recipes make_input_5_sp_layer \
        [--face-centers results/face_centers.dat] [--out input/input.dat]

Conventions (make_input.py:225-244, MUSCL_base.hpp:534-561): angular
momentum density l = Sigma (r x (omega x r)) / |r|^2, energy
E = Pi / (gam - 1) + Sigma |v|^2 / 2.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np


def read_face_centers(path: str | Path = "results/face_centers.dat") -> np.ndarray:
    """results/face_centers.dat: one whitespace-separated row of 3 values per face."""
    vals = np.array(Path(path).read_text().split(), dtype=np.float64)
    return vals.reshape(-1, 3)


def format_face_centers(unit_centers: np.ndarray) -> str:
    """The text of results/face_centers.dat for the given unit face centres,
    as the C++ writer prints it (setprecision(15), default float format,
    MUSCL_geometry.hpp:1069-1081)."""
    return "".join(f"{x:.15g} {y:.15g} {z:.15g}\n" for x, y, z in np.asarray(unit_centers, dtype=np.float64))


def _row_norms(R: np.ndarray) -> np.ndarray:
    """np.linalg.norm(R[i]) for every row (the reference's per-row norm: the
    square root of the row's dot product with itself)."""
    return np.sqrt(np.fromiter((r.dot(r) for r in R), dtype=np.float64, count=len(R)))


def _l_and_v(face_centers: np.ndarray, rho: np.ndarray, omega: np.ndarray, v_unit_cross: bool):
    """Per face: l = rho R x (omega x R) / |R|^2 and v = omega x R / |R|
    (v_unit_cross: v = omega x (R / |R|), the cos-bell and constant-entropy
    forms)."""
    R = np.asarray(face_centers, dtype=np.float64)
    omega = np.asarray(omega, dtype=np.float64)
    n = _row_norms(R)
    om = np.broadcast_to(omega, R.shape)
    oxr = np.cross(om, R)
    l = rho[:, None] * np.cross(R, oxr) / (n * n)[:, None]
    if v_unit_cross:
        v = np.cross(om, R / n[:, None])
    else:
        v = oxr / n[:, None]
    return l, v


def make_input_4(face_centers: np.ndarray) -> np.ndarray:
    """Isothermal (dim 4) solid-body rotation omega = 2 z with the balanced
    density rho = exp(-|omega|^2 sin^2(latitude) / 2) (make_input.py:6-38)."""
    fc = np.asarray(face_centers, dtype=np.float64)
    omega = np.array([0, 0, 2])
    r = np.sqrt(fc[:, 1] ** 2 + fc[:, 2] ** 2 + fc[:, 0] ** 2)
    rho = np.exp(-1 / 2 * (np.linalg.norm(omega) ** 2) * np.sin(-np.arccos(fc[:, 2] / r) + np.pi / 2) ** 2)
    l = np.empty((len(fc), 3))
    for i, R in enumerate(fc):
        l[i] = rho[i] * np.cross(R, np.cross(omega, R)) / (np.linalg.norm(R) ** 2)
    return np.column_stack([rho, l])


def make_input_4_cos_bell(face_centers: np.ndarray) -> np.ndarray:
    """Isothermal cosine bell rho = 1 + 10 cos(2.2 sqrt(theta^2 + phi^2)) in
    |lat|, |lon| < pi/6, rotating with omega = 2 z there and at rest
    elsewhere (make_input.py:40-74)."""
    fc = np.asarray(face_centers, dtype=np.float64)
    theta = -np.arccos(fc[:, 2]) + np.pi / 2
    phi = np.arctan2(fc[:, 1], fc[:, 0])
    rho = np.ones(len(fc))
    l = np.empty((len(fc), 3))
    for i, R in enumerate(fc):
        omega = np.array([0, 0, 0])
        if abs(theta[i]) < np.pi / 6 and abs(phi[i]) < np.pi / 6:
            rho[i] = 1 + 10 * np.cos(2.2 * np.sqrt(theta[i] ** 2 + phi[i] ** 2))
            omega = np.array([0, 0, 2])
        l[i] = rho[i] * np.cross(R, np.cross(omega, R)) / (np.linalg.norm(R) ** 2)
    return np.column_stack([rho, l])


def make_input_5(face_centers: np.ndarray) -> np.ndarray:
    """Adiabatic fluid at rest, rho = 1, with pressure 5 in a polar cap
    (|lat - pi/2| < 0.1) and 50 in a disc of radius 1/3 around (lat 0.3,
    lon 0.5), 1 elsewhere; gam3d 4/3 (make_input.py:78-143)."""
    fc = np.asarray(face_centers, dtype=np.float64)
    gam0 = 4.0 / 3
    gam = 2 - 1 / gam0
    N = len(fc)
    rho = np.ones(N)
    omega = np.array([0, 0, 0])
    p = np.ones(N)
    nrm = np.linalg.norm(fc, axis=1)
    theta = -np.arccos(fc[:, 2] / nrm) + np.pi / 2
    phi = np.arctan2(fc[:, 1] / nrm, fc[:, 0] / nrm)
    a = 1
    R0 = a / 3
    theta_c, phi_c = 0.3, 0.5
    r = a * np.arccos(np.sin(theta_c) * np.sin(theta) + np.cos(theta) * np.cos(theta_c) * np.cos(phi - phi_c))
    p[np.abs(theta - np.pi / 2) < 0.1] = 5
    p[r < R0] = 50
    l, v = _l_and_v(fc, rho, omega, v_unit_cross=False)
    vn = np.linalg.norm(v, axis=1)
    E = 1 / (gam - 1) * p + rho * vn * vn / 2
    return np.column_stack([rho, l, E])


def make_input_5_sp_layer(face_centers: np.ndarray) -> np.ndarray:
    """Spreading-layer equilibrium (the reference's active recipe): rotation
    omega = 0.01 z, rho_0 = 1/130, c_s = 2e-3, p_0 = c_s^2 rho_0 / gam;
    rho = rho_0 (1 + (gam-1)/2 M_0^2 sin^2 theta)^(1/(gam-1)) and p =
    p_0 (...)^(gam/(gam-1)), M_0 = |omega| / a_0 (make_input.py:145-244).
    Its input.dat is written with float_format "%.15f" (RECIPE_FLOAT_FORMAT)."""
    fc = np.asarray(face_centers, dtype=np.float64)
    gam0 = 4.0 / 3
    gam = 2 - 1 / gam0
    V_conv = 1
    N = len(fc)
    rho = np.ones(N)
    c_s = 2 * 10 ** (-3) / V_conv
    omega_ns = 0
    omega = np.array([0, 0, 0.01]) / V_conv
    rho_0 = rho[0] / 130
    p_0 = c_s ** 2 * rho_0 / gam
    a_0 = np.sqrt(gam * p_0 / rho_0)
    M_0 = np.linalg.norm(omega) / a_0
    theta = np.arccos(fc[:, 2] / np.linalg.norm(fc, axis=1))
    rho = rho_0 * (1 + (gam - 1) / 2 * M_0 ** 2 * np.sin(theta) ** 2) ** (1 / (gam - 1))
    p = p_0 * (1 + (gam - 1) / 2 * M_0 ** 2 * np.sin(theta) ** 2) ** (gam / (gam - 1))
    l, v = _l_and_v(fc, rho, omega, v_unit_cross=False)
    E = 1 / (gam - 1) * p + rho * ((np.linalg.norm(v, axis=1) ** 2) / 2
                                   - np.ones(N) * omega_ns ** 2 * (np.sin(theta) ** 2) / 2)
    return np.column_stack([rho, l, E])


def make_input_5_cos_bell(face_centers: np.ndarray) -> np.ndarray:
    """Cosine bell rho = 1 + 0.5 cos(pi r / R0) within R0 = 1/3 of (lat 0,
    lon 3 pi/2) on solid-body rotation omega = 0.5 z, p = 1 + |omega|^2 rho
    sin^2(lat) / 2, gam = 1.4 (make_input.py:249-291)."""
    fc = np.asarray(face_centers, dtype=np.float64)
    gam = 1.4
    N = len(fc)
    theta = -np.arccos(fc[:, 2]) + np.pi / 2
    phi = np.arctan2(fc[:, 1], fc[:, 0])
    omega = np.array([0, 0, 0.5])
    rho = np.ones(N)
    a = 1
    R0 = a / 3
    r = a * np.arccos(np.sin(0) * np.sin(theta) + np.cos(theta) * np.cos(0) * np.cos(phi - np.pi * 3 / 2))
    inside = r < R0
    rho[inside] = 1 + 0.5 * np.cos(np.pi * r[inside] / R0)
    l, v = _l_and_v(fc, rho, omega, v_unit_cross=True)
    p = 1 + (np.linalg.norm(omega) ** 2 * rho / 2 * np.sin(-np.arccos(fc[:, 2])) ** 2)
    vn = np.linalg.norm(v, axis=1)
    E = 1 / (gam - 1) * p + rho * vn * vn / 2
    return np.column_stack([rho, l, E])


def make_input_5_const_entr(face_centers: np.ndarray) -> np.ndarray:
    """Constant-entropy rotating equilibrium, omega = 5 z, rho_0 = p_0 = 1:
    rho = (1 + (gam-1)/2 M_0^2 sin^2 theta)^(1/(gam-1)), p = (...)^(gam/(gam-1))
    with theta = -arccos(z / |r|) (make_input.py:293-334)."""
    fc = np.asarray(face_centers, dtype=np.float64)
    gam0 = 4 / 3
    gam = 2 - 1 / gam0
    theta = -np.arccos((fc[:, 2]) / np.linalg.norm(fc, axis=1))
    omega = np.array([0, 0, 5])
    rho_0 = 1
    p_0 = 1
    a_0 = np.sqrt(gam * p_0 / rho_0)
    M_0 = np.linalg.norm(omega) / a_0
    rho = rho_0 * (1 + (gam - 1) / 2 * M_0 ** 2 * np.sin(theta) ** 2) ** (1 / (gam - 1))
    p = p_0 * (1 + (gam - 1) / 2 * M_0 ** 2 * np.sin(theta) ** 2) ** (gam / (gam - 1))
    l, v = _l_and_v(fc, rho, omega, v_unit_cross=True)
    vn = np.linalg.norm(v, axis=1)
    E = 1 / (gam - 1) * p + rho * vn * vn / 2
    return np.column_stack([rho, l, E])


RECIPES = {
    "make_input_4": make_input_4,
    "make_input_4_cos_bell": make_input_4_cos_bell,
    "make_input_5": make_input_5,
    "make_input_5_sp_layer": make_input_5_sp_layer,
    "make_input_5_cos_bell": make_input_5_cos_bell,
    "make_input_5_const_entr": make_input_5_const_entr,
}
# the float format each recipe's writer call passes (None: full precision)
RECIPE_FLOAT_FORMAT = {"make_input_5_sp_layer": "%.15f"}


def format_input_dat(U: np.ndarray, float_format: str | None = None) -> str:
    """The text of input/input.dat as the reference's writer produces it
    (space-separated, no index or header, one row per face): each value in
    float_format, or at full round-trip precision when it is None."""
    fmt = (lambda x: float_format % x) if float_format else (lambda x: repr(float(x)))
    return "".join(" ".join(fmt(x) for x in row) + "\n" for row in np.asarray(U, dtype=np.float64))


def write_input_dat(path: str | Path, U: np.ndarray, float_format: str | None = None) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_text(format_input_dat(U, float_format))


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description="write input/input.dat with one of the reference's recipes")
    ap.add_argument("recipe", choices=list(RECIPES))
    ap.add_argument("--face-centers", default="results/face_centers.dat")
    ap.add_argument("--out", default="input/input.dat")
    a = ap.parse_args(argv)
    U = RECIPES[a.recipe](read_face_centers(a.face_centers))
    write_input_dat(a.out, U, RECIPE_FLOAT_FORMAT.get(a.recipe))
    print(f"{a.out}: {len(U)} faces x {U.shape[1]} fields ({a.recipe})", file=sys.stderr)


if __name__ == "__main__":
    main()
