"""GPU checks of the tangent-linear model and the discrete adjoint of the
FP64 step (splash_tlm_run / splash_adjoint_* through the C ABI).

* The adjoint's forward run and the TLM's values are bit-identical to the
  FP64 solver (same kernels bodies, -fmad=false).
* TLM vs central finite differences of the forward run, with the
  difference step small enough that no limiter kink is crossed (state
  directions) or h = 1e-6 (parameter directions).
* Adjoint vs TLM: <lambda, J d> == <J^T lambda, d> to 1e-10 relative, for
  several checkpoint intervals (recomputation across interval boundaries).
* Loss gradient (1/2 sum area (Sigma - Sigma*)^2) vs finite differences.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import mesh_of

pytestmark = pytest.mark.gpu

GAM = 2 - 1 / (4 / 3)
DT = 5e-4
THETA = np.array([1e-2, 0.1, 0.5])  # accretion_rate, tilt_angle, omega_acc_abs


def _setup(level=3, solver=2, friction=True, accretion=True, seed=4):
    import splash_gb300 as sg

    mesh = mesh_of("hex", level)
    g = sg.Geometry(mesh)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), GAM, seed=seed)
    params = sg.SolverParams(accretion_rate=THETA[0], e_acc=0.5, omega_acc_abs=THETA[2], tilt_angle=THETA[1],
                             acc_width=0.1, alpha=1e-6, friction_on=friction)
    base = sg.Solver(mesh, U0, 5, GAM, 0.0, accretion, params=params, solver=solver, precision=sg.PREC_FP64)
    return sg, base, U0, g["area"].copy()


def _direction(rng, U0, scale_theta=1.0):
    """Random direction with per-field scales of U0 (a relative perturbation)."""
    scale = np.maximum(np.abs(U0).max(axis=0), 1e-3)
    dU = rng.normal(size=U0.shape) * scale
    dth = rng.normal(size=3) * np.array([1e-2, 0.1, 0.5]) * scale_theta
    return dU, dth


def test_adjoint_forward_and_tlm_values_match_the_solver():
    sg, base, U0, _ = _setup()
    ref = sg.Solver(sg.Mesh(0, 3), U0, 5, GAM, 0.0, True, params=base.params, solver=2, precision=sg.PREC_FP64)
    ref.do_steps(12, DT)
    Uref = ref.get_state()
    adj = sg.Adjoint(base, checkpoint_every=5)
    Uf = adj.forward(U0, THETA, 12, DT)
    assert np.array_equal(Uf, Uref)
    rng = np.random.default_rng(0)
    dU, dth = _direction(rng, U0)
    Ut, dUt = adj.tlm(U0, THETA, dU, dth, 12, DT)
    assert np.array_equal(Ut, Uref)
    assert np.isfinite(dUt).all() and np.abs(dUt).max() > 0
    assert adj.error_word() == 0
    info = adj.info()
    assert info["steps"] == 12 and info["clipped_steps"] == 0


def _noisy(U0, seed=5, amp=1e-3):
    """U0 with relative noise on Sigma and Pi, so no field is exactly uniform
    anywhere (the limited reconstruction has no derivative at a uniform
    state: there w + pp phi(pm / pp) bmd is positively homogeneous, not
    linear, in a perturbation)."""
    rng = np.random.default_rng(seed)
    U = U0.copy()
    U[:, 0] *= 1 + amp * rng.uniform(-1, 1, len(U))
    U[:, 4] *= 1 + amp * rng.uniform(-1, 1, len(U))
    return U


@pytest.mark.parametrize("solver,friction", [(1, True), (2, True), (3, True), (2, False)])
def test_tlm_matches_central_differences(solver, friction):
    """State directions: the limiters make the map rough at grid scale (a
    perturbation of relative size 1e-7 already crosses limiter kinks at a
    few faces), so the difference step is 1e-9 over two steps, where central
    differences resolve the derivative to round-off."""
    sg, base, U0, _ = _setup(solver=solver, friction=friction)
    U0 = _noisy(U0)
    adj = sg.Adjoint(base, checkpoint_every=10)
    n = 2
    rng = np.random.default_rng(solver)
    for _ in range(2):
        dU, _ = _direction(rng, U0)
        _, dUt = adj.tlm(U0, THETA, dU, None, n, DT)
        h = 1e-9
        fd = (adj.forward(U0 + h * dU, THETA, n, DT) - adj.forward(U0 - h * dU, THETA, n, DT)) / (2 * h)
        err = np.linalg.norm(fd - dUt) / np.linalg.norm(dUt)
        assert err < 1e-6, err


@pytest.mark.parametrize("solver,friction", [(1, True), (2, True), (3, True), (2, False)])
def test_parameter_tlm_matches_central_differences(solver, friction):
    """Parameter directions perturb the source proportionally to its own
    profile and stay in the differentiable regime: h = 1e-6, 10 steps."""
    sg, base, U0, _ = _setup(solver=solver, friction=friction)
    adj = sg.Adjoint(base, checkpoint_every=10)
    n = 10
    rng = np.random.default_rng(20 + solver)
    for dth in [np.array([1e-2, 0, 0]), np.array([0, 0.1, 0]), np.array([0, 0, 0.5]),
                rng.normal(size=3) * np.array([1e-2, 0.1, 0.5])]:
        _, dUt = adj.tlm(U0, THETA, None, dth, n, DT)
        h = 1e-6
        fd = (adj.forward(U0, THETA + h * dth, n, DT) - adj.forward(U0, THETA - h * dth, n, DT)) / (2 * h)
        err = np.linalg.norm(fd - dUt) / np.linalg.norm(dUt)
        assert err < 2e-5, (dth, err)


@pytest.mark.parametrize("K", [1, 4, 16])
@pytest.mark.parametrize("solver", [1, 2, 3])
def test_adjoint_dot_product_with_tlm(K, solver):
    """<lambda, J d> (TLM) == <J^T lambda, d> (adjoint), 16 steps."""
    sg, base, U0, _ = _setup(solver=solver, friction=(solver != 1))
    adj = sg.Adjoint(base, checkpoint_every=K)
    n = 16
    rng = np.random.default_rng(10 * K + solver)
    adj.forward(U0, THETA, n, DT)
    lam = rng.normal(size=U0.shape)
    gU, gth = adj.backward(lam)
    for _ in range(3):
        dU, dth = _direction(rng, U0)
        _, dUt = adj.tlm(U0, THETA, dU, dth, n, DT)
        lhs = float(np.sum(lam * dUt))
        rhs = float(np.sum(gU * dU) + np.dot(gth, dth))
        # relative to the magnitude of the summed terms (the sum may cancel)
        assert abs(lhs - rhs) <= 1e-10 * float(np.abs(lam * dUt).sum()), (lhs, rhs)


def test_parameter_gradients_match_tlm():
    """Each theta component separately: adjoint gradient vs TLM along e_i."""
    sg, base, U0, _ = _setup(friction=False)
    adj = sg.Adjoint(base, checkpoint_every=8)
    n = 16
    rng = np.random.default_rng(3)
    adj.forward(U0, THETA, n, DT)
    lam = rng.normal(size=U0.shape)
    _, gth = adj.backward(lam)
    for i in range(3):
        e = np.zeros(3)
        e[i] = 1.0
        _, dUt = adj.tlm(U0, THETA, None, e, n, DT)
        ref = float(np.sum(lam * dUt))
        assert abs(gth[i] - ref) <= 1e-9 * abs(ref), (i, gth[i], ref)


def test_loss_gradient_matches_finite_differences():
    """The loss of splash_adjoint_run: directional derivatives of the
    adjoint gradient vs the TLM (30 steps) and vs central differences (3
    steps on a nowhere-uniform state, h = 1e-8; parameter directions over
    30 steps, h = 1e-6)."""
    sg, base, U0, area = _setup(level=4)
    adj = sg.Adjoint(base, checkpoint_every=10)
    rng = np.random.default_rng(7)
    for n, Ustart, h, theta_only in [(30, U0, 1e-6, True), (3, _noisy(U0), 1e-8, False)]:
        target = adj.forward(Ustart, np.array([2e-2, 0.3, 0.5]), n, DT)[:, 0].copy()
        L, gU, gth = adj.run(Ustart, THETA, n, DT, target)
        Uf = adj.forward(Ustart, THETA, n, DT)
        assert abs(L - 0.5 * np.sum(area * (Uf[:, 0] - target) ** 2)) <= 1e-12 * L
        for _ in range(3):
            dU, dth = _direction(rng, Ustart)
            if theta_only:
                dU = np.zeros_like(dU)
            g_adj = float(np.sum(gU * dU) + np.dot(gth, dth))
            _, dUt = adj.tlm(Ustart, THETA, dU, dth, n, DT)
            g_tlm = float(np.sum(area * (Uf[:, 0] - target) * dUt[:, 0]))
            Lp, _, _ = adj.run(Ustart + h * dU, THETA + h * dth, n, DT, target)
            Lm, _, _ = adj.run(Ustart - h * dU, THETA - h * dth, n, DT, target)
            g_fd = (Lp - Lm) / (2 * h)
            assert abs(g_adj - g_tlm) <= 1e-10 * abs(g_tlm)
            assert abs(g_adj - g_fd) <= 1e-5 * abs(g_fd), (n, g_adj, g_fd)


def test_torch_function_matches_adjoint():
    torch = pytest.importorskip("torch")
    from splash_gb300.torch_adjoint import rollout

    sg, base, U0, area = _setup()
    adj = sg.Adjoint(base, checkpoint_every=4)
    n = 8
    U0t = torch.tensor(U0, requires_grad=True)
    tht = torch.tensor(THETA, requires_grad=True)
    Uf = rollout(adj, U0t, tht, n, DT)
    w = torch.tensor(np.random.default_rng(1).normal(size=U0.shape))
    (Uf * w).sum().backward()
    adj.forward(U0, THETA, n, DT)
    gU, gth = adj.backward(w.numpy())
    assert np.array_equal(U0t.grad.numpy(), gU)
    assert np.array_equal(tht.grad.numpy(), gth)


def test_adjoint_rejects_mixed_base():
    import splash_gb300 as sg

    mesh = mesh_of("hex", 3)
    g = sg.Geometry(mesh)
    U0 = sg.initial_conditions.rotating_blob(g.unit_face_centers(), GAM, seed=0)
    s = sg.Solver(mesh, U0, 5, GAM, 0.0, False, solver=2, precision=sg.PREC_MIXED)
    with pytest.raises(sg.SplashError):
        sg.Adjoint(s)


@pytest.mark.parametrize("solver", [1, 2, 3])
def test_branch_tape_record_replay_compare(solver):
    """splash_adjoint_branch_tape: recorded at x the run is the FP64
    forward bit for bit; replayed at x it is again, with no replayed
    decision contradicted; compared at x it departs nowhere, and compared at
    x + h d it is the plain forward at that point bit for bit and counts the
    (face, launch) evaluations whose branch path departs from x's: more at
    h = 1e-4 than at h = 1e-9.  On a nowhere-uniform state over 2 steps the
    crossings at h = 1e-9 are harmless (the kinks are continuous), and
    central differences of the loss match the adjoint to 1e-5."""
    sg, base, U0, area = _setup(solver=solver)
    U0 = _noisy(U0)
    n = 2
    adj = sg.Adjoint(base, checkpoint_every=1)
    target = adj.forward(U0, np.array([2e-2, 0.3, 0.5]), n, DT)[:, 0].copy()
    loss, gU, gth = adj.run(U0, THETA, n, DT, target)
    Uf = adj.forward(U0, THETA, n, DT)
    Ur, _ = adj.branch_tape(U0, THETA, n, "record")
    assert np.array_equal(Ur, Uf)
    Ux, flips = adj.branch_tape(U0, THETA, n, "replay")
    assert np.array_equal(Ux, Uf) and flips == 0
    Uc, dep = adj.branch_tape(U0, THETA, n, "compare")
    assert np.array_equal(Uc, Uf) and dep == 0

    def L(U):
        return 0.5 * float(np.sum(area * (U[:, 0] - target) ** 2))

    rng = np.random.default_rng(solver)
    dU, dth = _direction(rng, U0)
    g = float(np.sum(gU * dU) + np.dot(gth, dth))
    Ub, d_big = adj.branch_tape(U0 + 1e-4 * dU, THETA + 1e-4 * dth, n, "compare")
    assert np.array_equal(Ub, adj.forward(U0 + 1e-4 * dU, THETA + 1e-4 * dth, n, DT))
    h = 1e-9
    Up, dp = adj.branch_tape(U0 + h * dU, THETA + h * dth, n, "compare")
    Um, dm = adj.branch_tape(U0 - h * dU, THETA - h * dth, n, "compare")
    assert d_big > dp, (d_big, dp)
    fd = (L(Up) - L(Um)) / (2 * h)
    assert abs(fd - g) <= 1e-5 * abs(g), (solver, fd, g, dp, dm)
