"""Device-coded forms beyond the diffusion flux, against the oracle: a flux linear in
(alpha, beta, gamma) (the advection-diffusion tutorial's q = nu u - D grad u), and condition and
source values that depend on t through a factor exp(a (t - t0)) or 1 + a (t - t0) + b (t - t0)^2
(the annulus tutorial's u = 50 (1 - exp(-t/2)), the Brusselator's boundary values).  RHS within
1e-12 of the term scale; adaptive Tsit5 within 1e-8 of max|u| with the same step counts."""
import numpy as np
import pytest

import fvm_oracle as O
from problems import (advection_diffusion, annulus_time_dirichlet, api_problem, brusselator_phi,
                      brusselator_phi_exact, oracle_problem, parity_error, rhs_term_scale, time_forms_rect)

pytestmark = pytest.mark.gpu


def test_advection_diffusion_rhs(gpu_lib):
    import fvmgpu as F

    spec = advection_diffusion(121)
    oprob = oracle_problem(spec)
    prob = api_problem(spec)
    assert prob.info()["linear"] == 1
    rng = np.random.default_rng(31)
    for u in (spec.u0, spec.u0 + rng.standard_normal(spec.tri.num_points)):
        ref = O.fvm_eqs(oprob, u, 0.0)
        scale = rhs_term_scale(oprob, u, 0.0)
        for cons in (False, True):
            du = F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0, conservative=cons)
            assert parity_error(du, ref, scale) <= 1e-12, cons
    with pytest.raises(ValueError):  # the per-triangle path takes diffusion fluxes only
        F.fvm_eqs(np.zeros_like(spec.u0), spec.u0.copy(), prob, 0.0, force_triangle=True)


def test_advection_diffusion_solve(gpu_lib):
    import fvmgpu as F

    spec = advection_diffusion(61)
    spec.tf = 50.0
    prob = api_problem(spec)
    saveat = [0.0, 10.0, 25.0, 50.0]
    sol = F.solve(prob, F.Tsit5(), saveat=saveat)
    oprob = oracle_problem(spec)
    cb = lambda u, t: O.update_dirichlet_nodes(oprob, u, t)  # noqa: E731
    ref, st = O.tsit5_solve(lambda u, t: O.fvm_eqs(oprob, u, t), spec.u0, 0.0, spec.tf, saveat, callback=cb)
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    err = np.max(np.abs(np.array(sol.u) - ref)) / np.max(np.abs(ref))
    assert err < 1e-8, err
    # mass is carried to +x by nu = (0.05, 0): the first moment grows
    P = spec.tri.points
    assert np.sum(P[:, 0] * sol.u[-1]) > np.sum(P[:, 0] * sol.u[1]) > 0


@pytest.mark.parametrize("make", [annulus_time_dirichlet, brusselator_phi, time_forms_rect])
def test_time_dependent_rhs_and_dirichlet(gpu_lib, make):
    """fvm_eqs!(du, u, p, t) and update_dirichlet_nodes!(u, p, t) at times inside and outside
    [t0, tf]: the time factors are evaluated at the call's t."""
    import fvmgpu as F

    spec = make()
    oprob = oracle_problem(spec)
    prob = api_problem(spec)
    assert prob.info()["linear"] == 1 and len(prob.time_factors) >= 1
    rng = np.random.default_rng(7)
    u = spec.u0 + 0.1 * rng.standard_normal(spec.tri.num_points)
    for t in (spec.t0, spec.t0 + 0.3 * (spec.tf - spec.t0), spec.tf, spec.tf + 0.7):
        ref = O.fvm_eqs(oprob, u, t)
        scale = rhs_term_scale(oprob, u, t)
        for cons in (False, True):
            du = F.fvm_eqs(np.zeros_like(u), u.copy(), prob, t, conservative=cons)
            assert parity_error(du, ref, scale) <= 1e-12, (t, cons)
            if not cons:  # page-locked host arrays: the one-launch path, b(t) formed first
                u_pin, du_pin = F._lib.host_empty(u.shape), F._lib.host_empty(u.shape)
                u_pin[:] = u
                F.fvm_eqs(du_pin, u_pin, prob, t)
                assert np.array_equal(du_pin, du), t
        if oprob.conds.dirichlet_nodes:
            got = F.update_dirichlet_nodes(u.copy(), prob, t)
            want = O.update_dirichlet_nodes(oprob, u, t)
            assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want)), t
    with pytest.raises(ValueError):  # the per-triangle path has no time factors
        F.fvm_eqs(np.zeros_like(u), u.copy(), prob, spec.t0, force_triangle=True)


def _annulus_coarse():
    spec = annulus_time_dirichlet(12, 48)
    spec.tf = 0.5
    return spec


def _annulus_short():
    spec = annulus_time_dirichlet()
    spec.tf = 0.2
    return spec


@pytest.mark.parametrize("make,saveat,tol", [(_annulus_coarse, 0.05, 1e-3), (_annulus_short, 0.02, 1e-9),
                                             (time_forms_rect, 0.25, 1e-3)])
def test_time_dependent_solve(gpu_lib, make, saveat, tol):
    """Adaptive Tsit5 with time-dependent values runs on the host-controlled loop (captured
    steps would replay one t) and re-evaluates the first-same-as-last derivative after each
    Dirichlet update whose values change: the oracle's step sequence and RHS count.  The
    tutorial-size annulus (1062 steps to t = 0.2) steps at the explicit method's stability
    limit, where the step-size controller amplifies rounding differences in the error estimate
    to the integration tolerance (5e-5 .. 3e-4 of max|u| at reltol 1e-3, over identical step
    counts): it is compared at abstol = reltol = 1e-9 (5e-12 apart); the coarse annulus and
    the four-factor rectangle at the default tolerances."""
    import fvmgpu as F

    spec = make()
    prob = api_problem(spec)
    tols = {} if tol == 1e-3 else {"abstol": tol, "reltol": tol}
    sol = F.solve(prob, F.Tsit5(), saveat=saveat, **tols)
    assert sol.stats["driver"] == "host"
    oprob = oracle_problem(spec)
    cb = lambda u, t: O.update_dirichlet_nodes(oprob, u, t)  # noqa: E731
    ref, st = O.tsit5_solve(lambda u, t: O.fvm_eqs(oprob, u, t), spec.u0, spec.t0, spec.tf, list(sol.t),
                            callback=cb, **tols)
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    assert sol.stats["nrhs"] == st["nrhs"]
    err = np.max(np.abs(np.array(sol.u) - ref)) / np.max(np.abs(ref))
    assert err < 1e-8, err


def test_annulus_inner_value_follows_its_time_factor(gpu_lib):
    """The annulus tutorial (tutorial size, final time 2, saveat 0.2, 10704 steps): the inner
    circle holds 50 (1 - exp(-t/2)) at the final step end; a save inside a step holds the value
    of that step's start (du = 0 on Dirichlet rows), at most one step (< 1e-3) behind."""
    import fvmgpu as F

    spec = annulus_time_dirichlet()
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), saveat=0.2)
    assert len(sol.u) == 11 and sol.stats["driver"] == "host"
    inner = np.linalg.norm(spec.tri.points, axis=1) < 0.2 + 1e-9
    g = lambda t: 50 * (1 - np.exp(-t / 2))  # noqa: E731
    assert np.allclose(sol.u[-1][inner], g(2.0), rtol=1e-14, atol=0)
    for t, u in zip(sol.t[1:-1], sol.u[1:-1]):
        lag = g(t) - u[inner]
        assert np.all(lag >= 0) and np.all(lag <= g(t) - g(t - 1e-3)), t


def test_brusselator_phi_converges_to_its_exact_solution(gpu_lib):
    """u = exp(-x - y - t/2) solves the Brusselator-Phi problem: the GPU solution at t = 1 on
    40 x 40 and 80 x 80 grids is within the discretisation error, which falls with h."""
    import fvmgpu as F

    errs = []
    for n in (40, 80):
        spec = brusselator_phi(n)
        prob = api_problem(spec)
        sol = F.solve(prob, F.Tsit5(), saveat=[spec.tf], abstol=1e-10, reltol=1e-10)
        P = spec.tri.points
        exact = brusselator_phi_exact(P[:, 0], P[:, 1], spec.tf)
        errs.append(np.max(np.abs(sol.u[-1] - exact)) / np.max(np.abs(exact)))
    assert errs[0] < 2e-3 and errs[1] < 0.5 * errs[0], errs


def test_time_dependence_rejections(gpu_lib):
    """Time factors need a linear problem; templates and batches take time-independent ones."""
    import fvmgpu as F
    from problems import nonlinear_rect

    spec = nonlinear_rect(12)
    spec.bc_fns = (lambda x, y, t, u, p: t * x,) + tuple(spec.bc_fns[1:])
    prob = api_problem(spec)
    with pytest.raises(F.UnsupportedFormError, match="linear"):
        prob.handle
    spec = annulus_time_dirichlet(8, 32)
    mesh = F.FVMGeometry(spec.tri)
    BCs = F.BoundaryConditions(mesh, tuple(spec.bc_fns), (F.Neumann, F.Dirichlet))
    with pytest.raises(F.UnsupportedFormError):  # templates call conditions with t = u = nothing
        tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=lambda x, y, p: 1.0, initial_condition=spec.u0,
                                   final_time=1.0)
        F.solve(tmpl, F.Tsit5(), saveat=[1.0])
