"""Initial conditions in the reference's conserved-variable convention.

The reference stores U = (Sigma, l_x, l_y, l_z, E) per face with the
angular-momentum density l = Sigma (r x v) (so that the solver's
v = (r x l) / (-Sigma), MUSCL_base.hpp:534-535) and the energy
E = Pi / (gam - 1) + Sigma |v|^2 / 2 (MUSCL_base.hpp:561, make_input.py:225-238),
with r the unit face centre.  This module is a pandas-free restatement of
that convention plus the seeded recipes of the benchmark workloads; it
writes input/input.dat in the layout test.cpp:54-77 reads.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np


def gam2d(gam3d: float) -> float:
    """2-D adiabatic index used by the solver (test.cpp:28)."""
    return 2 - 1 / gam3d


def to_conserved(r_unit: np.ndarray, sigma: np.ndarray, pi: np.ndarray, v: np.ndarray,
                 gam: float) -> np.ndarray:
    """Primitive (Sigma, Pi, tangential v) -> conserved U [F, 5]."""
    r = np.asarray(r_unit, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    # keep only the tangential part of v
    v = v - np.sum(v * r, axis=1)[:, None] * r
    l = sigma[:, None] * np.cross(r, v)
    e = pi / (gam - 1) + sigma * np.sum(v * v, axis=1) / 2
    return np.column_stack([sigma, l, e])


def _tangential(r: np.ndarray, w: np.ndarray) -> np.ndarray:
    return w - np.sum(w * r, axis=1)[:, None] * r


def rotating_blob(r_unit: np.ndarray, gam: float, seed: int = 0, omega: float = 0.3,
                  noise: float = 1e-3) -> np.ndarray:
    """Density blob on solid-body rotation: Sigma = 1 + 0.2 exp(-|x-c|^2/0.05)
    with c a seeded unit vector, Pi = Sigma^gam, v = omega z x r plus
    tangential Gaussian noise (the small plain-method workload)."""
    rng = np.random.default_rng(seed)
    c = rng.normal(size=3)
    c /= np.linalg.norm(c)
    d2 = np.sum((r_unit - c) ** 2, axis=1)
    sigma = 1 + 0.2 * np.exp(-d2 / 0.05)
    pi = sigma ** gam
    v = omega * np.cross(np.array([0.0, 0.0, 1.0]), r_unit)
    v = v + _tangential(r_unit, rng.normal(0.0, noise, size=r_unit.shape))
    return to_conserved(r_unit, sigma, pi, v, gam)


def quiet_noise(r_unit: np.ndarray, gam: float, seed: int = 1, amp: float = 1e-3) -> np.ndarray:
    """Sigma = 1 and Pi = 1 with uniform noise of amplitude amp, zero velocity
    (the accreting mid-size workload and the ensemble instances)."""
    rng = np.random.default_rng(seed)
    n = r_unit.shape[0]
    sigma = 1 + rng.uniform(-amp, amp, size=n)
    pi = 1 + rng.uniform(-amp, amp, size=n)
    return to_conserved(r_unit, sigma, pi, np.zeros_like(r_unit), gam)


def _real_ylm(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Real spherical harmonic (unnormalised associated Legendre via scipy)."""
    from scipy.special import lpmv

    x = np.cos(theta)
    p = lpmv(abs(m), l, x)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - abs(m)) / math.factorial(l + abs(m)))
    if m > 0:
        return math.sqrt(2) * norm * p * np.cos(m * phi)
    if m < 0:
        return math.sqrt(2) * norm * p * np.sin(-m * phi)
    return norm * p


def shear_layer(r_unit: np.ndarray, gam: float, seed: int = 2, u0: float = 0.5,
                width: float = 0.05, lmax: int = 8, amp: float = 1e-2) -> np.ndarray:
    """Equatorial shear layer: u_phi = u0 tanh(latitude / width); Sigma = 1 +
    amp * (random real Y_lm, l <= lmax, normalised to unit max); Pi = Sigma^gam."""
    rng = np.random.default_rng(seed)
    x, y, z = r_unit[:, 0], r_unit[:, 1], r_unit[:, 2]
    theta = np.arccos(np.clip(z, -1, 1))
    phi = np.arctan2(y, x)
    lat = np.pi / 2 - theta
    pert = np.zeros_like(z)
    for l in range(1, lmax + 1):
        for m in range(-l, l + 1):
            pert += rng.normal() * _real_ylm(l, m, theta, phi)
    pert /= max(np.max(np.abs(pert)), 1e-300)
    sigma = 1 + amp * pert
    pi = sigma ** gam
    e_phi = np.column_stack([-y, x, np.zeros_like(x)])
    nrm = np.linalg.norm(e_phi, axis=1)
    e_phi = e_phi / np.where(nrm > 0, nrm, 1)[:, None]
    v = (u0 * np.tanh(lat / width))[:, None] * e_phi
    return to_conserved(r_unit, sigma, pi, v, gam)


def write_input_dat(path: str | Path, U: np.ndarray) -> None:
    """input/input.dat: one row of dim values per face (test.cpp:54-77)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    with open(path, "w") as f:
        for row in np.asarray(U):
            f.write(" ".join(repr(float(v)) for v in row) + "\n")
