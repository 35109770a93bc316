"""CPU check of the bound behind the mixed update's FP32 pressure recovery
(csrc/step_mixed.cu, store_face_state): where the kinetic term
|r x l|^2 / (2 Sigma), evaluated in FP32 from the FP32-rounded state, is at
most E / 8, Pi = (E - KE) (gam - 1) is evaluated in plain FP32 instead of in
double-word arithmetic.  The subtraction then loses at most a factor 8/7,
so the FP32 result stays within a few units in the last place of its float.
The FP32 branch is restated here in numpy float32 (IEEE division, where the
device uses its 2-ulp approximate quotient: a difference of at most 2/7 ulp
in Pi) and compared with the same formula in float64 on the FP64 state."""
from __future__ import annotations

import numpy as np

GAM3D = 4.0 / 3.0
GAM = 2.0 - 1.0 / GAM3D  # gam2d, the bench workloads' adiabatic index


def _states(rng, n, ke_over_e):
    """n FP64 states (Sigma, l, E) at unit centres r with a chosen ratio of
    kinetic to total energy."""
    r = rng.normal(size=(n, 3))
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    sigma = 10.0 ** rng.uniform(-3, 1, n)
    # a tangential momentum-like l (perpendicular to r, as r x (Sigma v))
    t = np.cross(r, rng.normal(size=(n, 3)))
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    l = t * (10.0 ** rng.uniform(-3, 1, n))[:, None]
    ke = 0.5 * np.sum(np.cross(r, l) ** 2, axis=1) / sigma
    E = ke / ke_over_e
    return r, sigma, l, E


def _fp32_branch(r, sigma, l, E):
    f = np.float32
    r32 = r.astype(f)
    w0 = sigma.astype(f)
    l32 = l.astype(f)
    E32 = E.astype(f)
    c = np.cross(r32, l32).astype(f)
    ke = (f(0.5) * (np.sum(c * c, axis=1, dtype=f) / w0)).astype(f)
    take = ke <= f(0.125) * E32
    pi = ((E32 - ke) * f(GAM - 1.0)).astype(f)
    return take, pi


def test_fp32_pressure_within_a_few_ulp_below_one_eighth():
    rng = np.random.default_rng(5)
    worst = 0.0
    for ratio in (1e-6, 1e-3, 0.05, 0.1, 0.124):
        r, sigma, l, E = _states(rng, 200_000, ratio)
        take, pi = _fp32_branch(r, sigma, l, E)
        assert take.all(), "states below E/8 take the FP32 branch"
        exact = (E - 0.5 * np.sum(np.cross(r, l) ** 2, axis=1) / sigma) * (GAM - 1.0)
        ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
        err = np.abs(pi.astype(np.float64) - exact) / ulp
        worst = max(worst, float(err.max()))
    assert worst <= 4.0, f"FP32 recovery off by {worst:.2f} ulp"


def test_cancelling_states_take_the_double_word_branch():
    rng = np.random.default_rng(6)
    r, sigma, l, E = _states(rng, 100_000, 0.5)
    take, _ = _fp32_branch(r, sigma, l, E)
    assert not take.any()
