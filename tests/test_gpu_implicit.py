"""Implicit stepping on the device: the Jacobian-vector product and diagonal of fvm_eqs!
against the oracle's finite differences, and TR-BDF2 (simplified Newton, matrix-free
BiCGStab) against the oracle's TR-BDF2 with exact sparse solves."""
import numpy as np
import pytest

import fvm_oracle as O
from problems import (annulus_time_dirichlet, api_problem, mixed_annulus, nonlinear_rect, oracle_problem,
                      readme_diffusion, sine_diffusion)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", [lambda: sine_diffusion(24), mixed_annulus, lambda: nonlinear_rect(16)])
def test_jvp_against_oracle_directional_derivative(gpu_lib, make):
    """J(u) v on the operator path (linear forms, with the quadratic diagonal terms of
    mixed_annulus) and on the per-triangle path (D(u), quadratic Neumann, logistic source):
    central differences of the oracle's fvm_eqs!, 1e-7 of max|J v|."""
    import fvmgpu as F

    spec = make()
    prob = api_problem(spec)
    oprob = oracle_problem(spec)
    rng = np.random.default_rng(3)
    n = spec.tri.num_points
    for _ in range(2):
        u = np.asarray(spec.u0, dtype=np.float64) + 0.1 * rng.standard_normal(n)
        v = rng.standard_normal(n)
        got = F.jvp(prob, u, v)
        eps = 1e-5
        fd = (O.fvm_eqs(oprob, u + eps * v, 0.0) - O.fvm_eqs(oprob, u - eps * v, 0.0)) / (2 * eps)
        assert np.max(np.abs(got - fd)) <= 1e-7 * np.max(np.abs(fd)), np.max(np.abs(got - fd)) / np.max(np.abs(fd))


@pytest.mark.parametrize("make", [lambda: sine_diffusion(12), mixed_annulus, lambda: nonlinear_rect(10)])
def test_jacobian_diagonal_against_oracle(gpu_lib, make):
    import fvmgpu as F

    spec = make()
    prob = api_problem(spec)
    oprob = oracle_problem(spec)
    u = np.asarray(spec.u0, dtype=np.float64) + 0.05
    ent, n = O.jacobian_sparsity(spec.tri)
    J = O.colored_jacobian(lambda x, t: O.fvm_eqs(oprob, x, t), u, 0.0, ent, n)
    want = J.diagonal()
    got = F.jacobian_diagonal(prob, u)
    assert np.max(np.abs(got - want)) <= 1e-6 * np.max(np.abs(want))


def _oracle_trbdf2(spec, saveat, affine, **kw):
    oprob = oracle_problem(spec)
    f = lambda u, t: O.fvm_eqs(oprob, u, t)  # noqa: E731
    ent, n = O.jacobian_sparsity(spec.tri)
    if affine:
        J = O.colored_jacobian(f, spec.u0, spec.t0, ent, n, affine=True)
        jac = lambda u, t: J  # noqa: E731
    else:
        jac = lambda u, t: O.colored_jacobian(f, u, t, ent, n)  # noqa: E731
    cb = (lambda u, t: O.update_dirichlet_nodes(oprob, u, t)) if oprob.conds.dirichlet_nodes else None
    return O.trbdf2_solve(f, jac, spec.u0, spec.t0, spec.tf, saveat, callback=cb, affine=affine, **kw)


def test_trbdf2_linear_matches_oracle(gpu_lib):
    """README diffusion (30 x 30) to t = 0.5, adaptive: the oracle's steps, solutions within
    1e-8 of max|u| (the device's Krylov solves stop at 1e-10 of the right-hand side)."""
    import fvmgpu as F

    spec = readme_diffusion(30)
    prob = api_problem(spec)
    saveat = [0.0, 0.05, 0.25, 0.5]
    sol = F.solve(prob, F.TRBDF2(), saveat=saveat)
    ref, st = _oracle_trbdf2(spec, saveat, affine=True)
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    assert sol.stats["newton_iters"] == st["newton"] and sol.stats["newton_failures"] == 0
    err = np.max(np.abs(np.array(sol.u) - ref)) / 50.0
    assert err < 1e-8, err


def test_trbdf2_fixed_step_matches_oracle(gpu_lib):
    import fvmgpu as F

    spec = sine_diffusion(24)
    spec.tf = 0.05
    prob = api_problem(spec)
    sol = F.solve(prob, F.TRBDF2(), dt=1e-3, adaptive=False, saveat=[0.0, 0.0125, 0.05])
    ref, st = _oracle_trbdf2(spec, [0.0, 0.0125, 0.05], affine=True, dt=1e-3, adaptive=False)
    assert sol.stats["naccept"] == st["naccept"] == 50
    err = np.max(np.abs(np.array(sol.u) - ref)) / np.max(np.abs(ref))
    assert err < 1e-9, err


def test_trbdf2_nonlinear_matches_oracle(gpu_lib):
    """Nonlinear forms (D(u), quadratic Neumann, logistic source) at tight tolerances: Newton
    iterations with the exact device JVP against the oracle's with a finite-difference
    Jacobian, both converged to the same stage equations."""
    import fvmgpu as F

    spec = nonlinear_rect(16)
    prob = api_problem(spec)
    saveat = [0.0, 0.005, 0.01]
    sol = F.solve(prob, F.TRBDF2(), saveat=saveat, abstol=1e-8, reltol=1e-8)
    ref, st = _oracle_trbdf2(spec, saveat, affine=False, abstol=1e-8, reltol=1e-8)
    assert abs(sol.stats["naccept"] - st["naccept"]) <= 2
    err = np.max(np.abs(np.array(sol.u) - ref)) / np.max(np.abs(ref))
    assert err < 1e-6, err


def test_trbdf2_takes_large_steps_on_a_stiff_problem(gpu_lib):
    """The annulus tutorial (time-dependent inner value, tutorial size, to t = 2) needs 10704
    Tsit5 steps at the default tolerances, at the explicit method's stability limit; TR-BDF2 is
    A-stable and takes about 300 (measured 297), set by accuracy alone, and agrees with a
    tight-tolerance Tsit5 solution to the integration tolerance."""
    import fvmgpu as F

    spec = annulus_time_dirichlet()
    prob = api_problem(spec)
    saveat = [0.0, 0.5, 1.0, 2.0]
    imp = F.solve(prob, F.TRBDF2(), saveat=saveat)
    assert imp.stats["naccept"] < 10704 // 20
    ref = F.solve(prob, F.Tsit5(), saveat=saveat, abstol=1e-9, reltol=1e-9)
    err = np.max(np.abs(np.array(imp.u) - np.array(ref.u))) / np.max(np.abs(ref.u))
    assert err < 1e-2, err
    inner = np.linalg.norm(spec.tri.points, axis=1) < 0.2 + 1e-9
    assert np.allclose(imp.u[-1][inner], 50 * (1 - np.exp(-1.0)), rtol=1e-13)


def test_trbdf2_on_a_template_matches_oracle(gpu_lib):
    """DiffusionEquation with TR-BDF2 (J = A): the oracle's TR-BDF2 on its own sparse assembly of
    A and b, the same steps, 1e-8 of max|u|."""
    import fvmgpu as F

    spec = sine_diffusion(30)
    mesh = F.FVMGeometry(spec.tri)
    BCs = F.BoundaryConditions(mesh, spec.bc_fns[0], F.Dirichlet)
    D = lambda x, y, p: spec.D(x, y, 0, 0, None)  # noqa: E731
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=D, initial_condition=spec.u0, final_time=0.02)
    saveat = [0.0, 0.01, 0.02]
    sol = F.solve(tmpl, F.TRBDF2(), saveat=saveat)
    conds = O.Conditions(spec.tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b, u0 = O.template_diffusion(spec.tri, conds, lambda x, y: D(x, y, None), spec.u0)
    ref, st = O.trbdf2_solve(lambda u, t: A @ u + b, lambda u, t: A, u0, 0.0, 0.02, saveat, affine=True)
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    got = np.array([row[:-1] for row in sol.u])
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err < 1e-8, err
