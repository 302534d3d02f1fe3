"""The discrete adjoint of the time-dependent templates (variant: differentiation).

D(x, y) of instance i is the P1 interpolant of exp(theta[:, i]).  Checked against the oracle:
the operator (oracle template assembly with that D, 1e-12 relative), the forward Tsit5 solve
(1e-10), the right-hand-side VJP (u_bar = A^T w to 1e-12; theta_bar against central finite
differences of the oracle right-hand side to 1e-7), and the gradient of
loss = sum (u(T) - u_obs)^2 against central finite differences of the oracle's forward solve
(max-norm error <= 1e-6 of the gradient's max-norm).  At the full workload (512 x 512, 200
steps of 1e-6, checkpoints every 20 steps) the gradient is checked on 32 random vertices
against central differences computed with the batched GPU forward solve.  Finite differences
of the loss are formed per vertex, sum (u+ - u-)(u+ + u- - 2 u_obs), so that the sum does not
cancel catastrophically."""
import numpy as np
import pytest

import fvm_oracle as O
from fvmgpu.meshes import triangulate_rectangle

pytestmark = pytest.mark.gpu


def fourier_field(P, seed, sigma, modes=16):
    """sigma * sum_m a_m cos(2 pi k_m . x + phi_m) / sqrt(modes / 2), seeded."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(modes)
    k = rng.integers(1, 5, size=(modes, 2))
    ph = rng.uniform(0, 2 * np.pi, modes)
    s = sum(a[m] * np.cos(2 * np.pi * (k[m, 0] * P[:, 0] + k[m, 1] * P[:, 1]) + ph[m]) for m in range(modes))
    return sigma * s / np.sqrt(modes / 2)


def diffusion_template(F, n):
    """DiffusionEquation on [0, 1]^2 (n x n points), zero Dirichlet, u0 a Gaussian bump."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, lambda x, y, t, u, p: 0.0 * x, F.Dirichlet)
    P = tri.points
    u0 = np.exp(-50 * ((P[:, 0] - 0.5) ** 2 + (P[:, 1] - 0.5) ** 2))
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=lambda x, y, p: 1.0 + 0.0 * x, initial_condition=u0,
                               final_time=1.0)
    return tri, tmpl


def oracle_operator(tri, theta):
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b, _ = O.template_diffusion(tri, conds, O.p1_field(tri, np.exp(theta)), np.zeros(tri.num_points))
    return A, b


def fd_loss_difference(up, um, obs):
    """loss(u+) - loss(u-) for loss = sum (u - obs)^2, per vertex."""
    return float(np.sum((up - um) * (up + um - 2 * obs)))


def test_operator_and_forward_match_oracle(gpu_lib):
    import fvmgpu as F

    tri, tmpl = diffusion_template(F, 14)
    n, B = tri.num_points, 3
    thetas = np.stack([np.log(0.5) + fourier_field(tri.points, s, 0.3) for s in range(B)], axis=1)
    adj = F.AdjointProblem(tmpl, batch=B).set_log_diffusion(thetas)
    u = np.random.default_rng(0).random((n, B))
    du = adj.rhs(u)
    dt, N = 2e-4, 12
    uT = adj.forward(np.ascontiguousarray(np.repeat(tmpl.u0[:, None], B, axis=1)), dt, N)
    for i in range(B):
        A, b = oracle_operator(tri, thetas[:, i])
        ref = A @ u[:, i] + b
        assert np.linalg.norm(du[:, i] - ref) <= 1e-12 * np.linalg.norm(ref)
        refT = O.template_ode_solve(A, b, tmpl.u0, dt, N)
        assert np.max(np.abs(uT[:, i] - refT)) <= 1e-10 * np.max(np.abs(refT))


def test_rhs_vjp_against_oracle(gpu_lib):
    import fvmgpu as F

    tri, tmpl = diffusion_template(F, 12)
    n = tri.num_points
    rng = np.random.default_rng(1)
    theta = np.log(0.7) + fourier_field(tri.points, 5, 0.4)
    adj = F.AdjointProblem(tmpl, batch=1).set_log_diffusion(theta[:, None].copy())
    u, w = rng.random((n, 1)), rng.standard_normal((n, 1))
    ub, tb = adj.rhs_vjp(u, w)
    A, _ = oracle_operator(tri, theta)
    assert np.linalg.norm(ub[:, 0] - A.T @ w[:, 0]) <= 1e-12 * np.linalg.norm(A.T @ w[:, 0])
    # directional derivative of <w, f(u, theta)> along a random direction, central differences
    d = rng.standard_normal(n)
    eps = 1e-5
    Ap, _ = oracle_operator(tri, theta + eps * d)
    Am, _ = oracle_operator(tri, theta - eps * d)
    fd = float(w[:, 0] @ ((Ap - Am) @ u[:, 0])) / (2 * eps)
    assert abs(float(tb[:, 0] @ d) - fd) <= 1e-7 * abs(fd)


def test_gradient_against_oracle_finite_differences(gpu_lib):
    import fvmgpu as F

    tri, tmpl = diffusion_template(F, 12)
    n = tri.num_points
    dt, N, K = 4e-4, 10, 3
    theta_true = np.log(0.6) + fourier_field(tri.points, 11, 0.4)
    A, b = oracle_operator(tri, theta_true)
    obs = O.template_ode_solve(A, b, tmpl.u0, dt, N)
    theta = np.log(0.6) + fourier_field(tri.points, 12, 0.2)
    adj = F.AdjointProblem(tmpl, batch=1).set_log_diffusion(theta[:, None].copy())
    loss, g, g0, st = adj.loss_and_grad(tmpl.u0[:, None].copy(), obs[:, None].copy(), dt, N, checkpoint_every=K)
    assert st["steps"] == N and st["checkpoints"] == (N + K - 1) // K
    A, b = oracle_operator(tri, theta)
    uT = O.template_ode_solve(A, b, tmpl.u0, dt, N)
    assert abs(loss[0] - np.sum((uT - obs) ** 2)) <= 1e-10 * loss[0]
    verts = np.random.default_rng(3).choice(n, size=32, replace=False)
    eps = 1e-4
    fd = np.empty(verts.size)
    for j, v in enumerate(verts):
        tp, tm = theta.copy(), theta.copy()
        tp[v] += eps
        tm[v] -= eps
        Ap, bp = oracle_operator(tri, tp)
        Am, bm = oracle_operator(tri, tm)
        up = O.template_ode_solve(Ap, bp, tmpl.u0, dt, N)
        um = O.template_ode_solve(Am, bm, tmpl.u0, dt, N)
        fd[j] = fd_loss_difference(up, um, obs) / (2 * eps)
    err = np.max(np.abs(g[verts, 0] - fd)) / np.max(np.abs(g[:, 0]))
    assert err <= 1e-6, err
    # d loss / d u0 along a random direction
    d = np.random.default_rng(4).standard_normal(n)
    e0 = 1e-4
    up = O.template_ode_solve(A, b, tmpl.u0 + e0 * d, dt, N)
    um = O.template_ode_solve(A, b, tmpl.u0 - e0 * d, dt, N)
    fd0 = fd_loss_difference(up, um, obs) / (2 * e0)
    assert abs(float(g0[:, 0] @ d) - fd0) <= 1e-7 * abs(fd0)


def test_checkpoint_interval_and_batching_do_not_change_the_gradient(gpu_lib):
    import fvmgpu as F

    tri, tmpl = diffusion_template(F, 16)
    n, B = tri.num_points, 4
    dt, N = 3e-4, 9
    thetas = np.stack([np.log(0.5) + fourier_field(tri.points, 20 + s, 0.3) for s in range(B)], axis=1)
    u0 = np.ascontiguousarray(np.repeat(tmpl.u0[:, None], B, axis=1))
    obs = np.ascontiguousarray(0.9 * u0)
    adj = F.AdjointProblem(tmpl, batch=B).set_log_diffusion(thetas)
    ref = None
    for K in (1, 4, 9, 50):
        loss, g, g0, _ = adj.loss_and_grad(u0, obs, dt, N, checkpoint_every=K)
        if ref is None:
            ref = (loss, g, g0)
        else:
            assert np.array_equal(loss, ref[0]) and np.max(np.abs(g - ref[1])) <= 1e-14 * np.max(np.abs(ref[1]))
    for i in (0, 3):
        one = F.AdjointProblem(tmpl, batch=1).set_log_diffusion(thetas[:, i:i + 1].copy())
        l1, g1, _, _ = one.loss_and_grad(u0[:, i:i + 1].copy(), obs[:, i:i + 1].copy(), dt, N, checkpoint_every=4)
        assert abs(l1[0] - ref[0][i]) <= 1e-13 * ref[0][i]
        assert np.max(np.abs(g1[:, 0] - ref[1][:, i])) <= 1e-12 * np.max(np.abs(ref[1][:, i]))
    # the pullback with uT_bar = 2 (u(T) - u_obs) is the loss gradient; the rrule wraps it
    uT, pb = F.solve_rrule(adj, thetas, u0, dt, N, checkpoint_every=4)
    tb, ub = pb(np.ascontiguousarray(2 * (uT - obs)))
    assert np.max(np.abs(tb - ref[1])) <= 1e-12 * np.max(np.abs(ref[1]))


def test_full_size_gradient_against_batched_finite_differences(gpu_lib):
    """512 x 512 mesh, 200 Tsit5 steps of dt = 1e-6, checkpoints every 20 steps; u_obs from a
    seeded true log-D field (log 0.4 plus 16 Fourier modes of amplitude 0.3); central
    differences on 32 random vertices, all 64 perturbed solves in one batched forward."""
    import fvmgpu as F

    tri, tmpl = diffusion_template(F, 512)
    n = tri.num_points
    dt, N, K = 1e-6, 200, 20
    # D stays below ~1: dt * (largest eigenvalue ~ 8 D / h^2) ~ 2, inside Tsit5's stability interval
    theta_true = np.log(0.4) + fourier_field(tri.points, 7, 0.3)
    theta = np.full(n, np.log(0.4))
    truth = F.AdjointProblem(tmpl, batch=1).set_log_diffusion(theta_true[:, None].copy())
    obs = truth.forward(tmpl.u0[:, None].copy(), dt, N)
    adj = F.AdjointProblem(tmpl, batch=1).set_log_diffusion(theta[:, None].copy())
    loss, g, _, st = adj.loss_and_grad(tmpl.u0[:, None].copy(), obs, dt, N, checkpoint_every=K)
    assert st["checkpoints"] == N // K and loss[0] > 0
    verts = np.random.default_rng(8).choice(n, size=32, replace=False)
    eps = 1e-4
    th = np.repeat(theta[:, None], 64, axis=1)
    th[verts, np.arange(32)] += eps
    th[verts, 32 + np.arange(32)] -= eps
    fdp = F.AdjointProblem(tmpl, batch=64).set_log_diffusion(np.ascontiguousarray(th))
    uT = fdp.forward(np.ascontiguousarray(np.repeat(tmpl.u0[:, None], 64, axis=1)), dt, N)
    fd = np.array([fd_loss_difference(uT[:, j], uT[:, 32 + j], obs[:, 0]) for j in range(32)]) / (2 * eps)
    err = np.max(np.abs(g[verts, 0] - fd)) / np.max(np.abs(g[:, 0]))
    assert err <= 1e-6, err
