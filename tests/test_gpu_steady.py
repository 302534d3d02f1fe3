"""Steady states on the device (SteadyFVMProblem with DynamicSS and NewtonRaphson, through
fvm_steady_solve / fvm_system_steady_solve) against the oracle's Newton steady solve with
exact sparse solves (oracle/fvm_oracle.py: steady_newton), on the reference tutorials'
steady problems: Laplace with an internal Dirichlet line, Helmholtz with Neumann values, mean
exit time on a disk, a nonlinear diffusivity and a coupled nonlinear system."""
import numpy as np
import pytest

import fvm_oracle as O
from fvmgpu.meshes import triangulate_disk, triangulate_rectangle
from problems import Spec, api_problem, oracle_problem

pytestmark = pytest.mark.gpu


def _oracle_steady(spec, **kw):
    oprob = oracle_problem(spec)
    f = lambda u, t: O.fvm_eqs(oprob, u, t)  # noqa: E731
    ent, n = O.jacobian_sparsity(spec.tri)
    jac = lambda u, t: O.colored_jacobian(f, u, t, ent, n)  # noqa: E731
    cb = (lambda u, t: O.update_dirichlet_nodes(oprob, u, t)) if oprob.conds.dirichlet_nodes else None
    u, it, _ = O.steady_newton(f, jac, spec.u0, spec.t0, O.fixed_rows(spec.tri, [oprob.conds]), callback=cb, **kw)
    return u, it


def laplace_internal_line(n=51) -> Spec:
    """docs/src/literate_tutorials/laplaces_equation_with_internal_dirichlet_conditions.jl: u = 0,
    100y, 100, 100y on the unit square's sides, u = 0 on the line x = 1/2, y <= 2/5, initial guess
    100y off the line (the tutorial refines its mesh around the line; here the lattice has a
    column of points on it)."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    P = tri.points
    line = np.nonzero((np.abs(P[:, 0] - 0.5) < 1e-12) & (P[:, 1] <= 0.4 + 1e-12))[0]
    bcs = (lambda x, y, t, u, p: 0.0 * x, lambda x, y, t, u, p: 100 * y, lambda x, y, t, u, p: 100.0 + 0.0 * x,
           lambda x, y, t, u, p: 100 * y)
    u0 = np.where((np.abs(P[:, 0] - 0.5) < 1e-12) & (P[:, 1] <= 0.4 + 1e-12), 0.0, 100 * P[:, 1])
    return Spec(tri, bcs, ("Dirichlet",) * 4, (None,) * 4, ic_fns=(lambda x, y, t, u, p: 0.0 * x,), ic_params=(None,),
                dirichlet_nodes={int(i): 0 for i in line}, D=lambda x, y, t, u, p: 1.0 + 0.0 * x, u0=u0,
                tf=np.inf)


def helmholtz(n=40) -> Spec:
    """docs/src/literate_tutorials/helmholtz_equation_with_inhomogeneous_boundary_conditions.jl:
    div grad u + u = 0 on [-1, 1]^2 with q.n = -1 on the boundary, initial guess 0."""
    tri = triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, n, n, single_boundary=True)
    return Spec(tri, (lambda x, y, t, u, p: -1.0 + 0.0 * x,), ("Neumann",), (None,),
                D=lambda x, y, t, u, p: 1.0 + 0.0 * x, S=lambda x, y, t, u, p: u, u0=np.zeros(tri.num_points),
                tf=np.inf)


def mean_exit_disk() -> Spec:
    """The mean exit time of a unit disk with D = 1 as the steady state of du/dt = div grad u + 1
    (docs/src/literate_tutorials/mean_exit_time.jl solves its problems this way): (1 - r^2)/4."""
    tri = triangulate_disk(3000, 128, seed=5)
    return Spec(tri, (lambda x, y, t, u, p: 0.0 * x,), ("Dirichlet",), (None,),
                D=lambda x, y, t, u, p: 1.0 + 0.0 * x, S=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                u0=np.zeros(tri.num_points), tf=np.inf)


def nonlinear_diffusivity(n=24) -> Spec:
    """div((1 + u^2) grad u) = 0 with u = x + y on the boundary of the unit square (the
    per-triangle path), initial guess 0 inside."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=True)
    return Spec(tri, (lambda x, y, t, u, p: x + y,), ("Dirichlet",), (None,),
                D=lambda x, y, t, u, p: 1.0 + u * u, u0=np.zeros(tri.num_points), tf=np.inf)


@pytest.mark.parametrize("method", ["newton", "dynamic"])
def test_laplace_internal_line_matches_oracle(gpu_lib, method):
    import fvmgpu as F

    spec = laplace_internal_line()
    steady = F.SteadyFVMProblem(api_problem(spec))
    alg = F.NewtonRaphson() if method == "newton" else F.DynamicSS(F.TRBDF2())
    sol = F.solve(steady, alg)
    ref, _ = _oracle_steady(spec)
    err = np.max(np.abs(sol.u - ref)) / 100.0
    # Newton stops at 1e-10 of max|f + u|; DynamicSS at reltol 1e-6 of it (|J^-1| <= 0.1 here)
    assert err < (1e-9 if method == "newton" else 1e-6), err
    assert sol.retcode == "Success" and sol.stats["method"] == method
    line = list(spec.dirichlet_nodes)
    assert np.all(sol.u[line] == 0.0)
    if method == "newton":
        assert sol.stats["iterations"] <= 2  # affine: one Newton step to the Krylov tolerance


def test_helmholtz_newton_then_dynamic(gpu_lib):
    """The tutorial's sequence: NewtonRaphson from 0, then DynamicSS(TRBDF2) from that solution,
    which stops after its first step."""
    import fvmgpu as F

    spec = helmholtz()
    prob = api_problem(spec)
    steady = F.SteadyFVMProblem(prob)
    sol = F.solve(steady, F.NewtonRaphson())
    ref, _ = _oracle_steady(spec)
    assert np.max(np.abs(sol.u - ref)) <= 1e-8 * np.max(np.abs(ref))
    prob.initial_condition[:] = sol.u
    sol2 = F.solve(steady, F.DynamicSS(F.TRBDF2()))
    assert sol2.stats["iterations"] == 1
    assert np.max(np.abs(sol2.u - ref)) <= 1e-6 * np.max(np.abs(ref))


def test_mean_exit_time_dynamic_ss(gpu_lib):
    import fvmgpu as F

    spec = mean_exit_disk()
    sol = F.solve(F.SteadyFVMProblem(api_problem(spec)), F.DynamicSS(F.TRBDF2(), abstol=1e-10, reltol=1e-10))
    ref, _ = _oracle_steady(spec)
    assert np.max(np.abs(sol.u - ref)) <= 1e-7 * np.max(ref)
    r2 = (spec.tri.points**2).sum(axis=1)
    assert np.max(np.abs(sol.u - (1 - r2) / 4)) <= 5e-3 * 0.25


@pytest.mark.parametrize("method", ["newton", "dynamic"])
def test_nonlinear_diffusivity_matches_oracle(gpu_lib, method):
    import fvmgpu as F

    spec = nonlinear_diffusivity()
    steady = F.SteadyFVMProblem(api_problem(spec))
    alg = F.NewtonRaphson() if method == "newton" else F.DynamicSS(F.TRBDF2(), abstol=1e-10, reltol=1e-10)
    sol = F.solve(steady, alg)
    ref, it = _oracle_steady(spec)
    assert np.max(np.abs(sol.u - ref)) <= 1e-8 * np.max(np.abs(ref))
    if method == "newton":
        assert abs(sol.stats["iterations"] - it) <= 1


def test_newton_not_converged_reports_the_last_iterate(gpu_lib):
    import fvmgpu as F

    spec = nonlinear_diffusivity(12)
    steady = F.SteadyFVMProblem(api_problem(spec))
    with pytest.raises(F.NotConvergedError) as ei:
        F.solve(steady, F.NewtonRaphson(max_iters=1))
    sol = ei.value.solution
    assert sol.retcode == "Failure" and sol.stats["iterations"] == 1 and np.all(np.isfinite(sol.u))


def test_time_stepping_an_infinite_final_time_is_refused(gpu_lib):
    import fvmgpu as F

    prob = api_problem(laplace_internal_line(11))
    with pytest.raises(ValueError, match="SteadyFVMProblem"):
        F.solve(prob, F.Tsit5())
    assert "SteadyFVMProblem with" in repr(F.SteadyFVMProblem(prob))


def _reaction_system(n=20):
    """u, v on the unit square with u = 1, v = 1/2 on the boundary, D_u = 1, D_v = 1/2 and the
    monotone cubic sources 4(v - u^3) and 4(u - v - v^3): a unique steady state, off the
    boundary values inside."""
    from test_gpu_system import SysSpec

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=True)
    comps = [dict(bc=(lambda x, y, t, u, p: 1.0 + 0.0 * x,), bcp=(None,), types=("Dirichlet",),
                  q=lambda x, y, t, a, b, g, p: (-a[0], -b[0]), S=lambda x, y, t, u, p: 4 * (u[1] - u[0] ** 3)),
             dict(bc=(lambda x, y, t, u, p: 0.5 + 0.0 * x,), bcp=(None,), types=("Dirichlet",),
                  q=lambda x, y, t, a, b, g, p: (-a[1] / 2, -b[1] / 2),
                  S=lambda x, y, t, u, p: 4 * (u[0] - u[1] - u[1] ** 3))]
    u0 = np.stack([np.ones(tri.num_points), np.full(tri.num_points, 0.5)])
    return SysSpec(tri, comps, u0, tf=np.inf)


@pytest.mark.parametrize("method", ["newton", "dynamic"])
def test_system_steady_state_matches_oracle(gpu_lib, method):
    import fvmgpu as F

    spec = _reaction_system()
    osys, sys_ = spec.oracle(), spec.api()
    N = 2
    f = lambda x, t: O.system_fvm_eqs(osys, x.reshape(-1, N).T, t).T.ravel()  # noqa: E731
    ent, nn = O.jacobian_sparsity(spec.tri, N)
    jac = lambda x, t: O.colored_jacobian(f, x, t, ent, nn)  # noqa: E731
    cb = lambda x, t: O.system_update_dirichlet_nodes(osys, x.reshape(-1, N).T, t).T.ravel()  # noqa: E731
    ref, it, _ = O.steady_newton(f, jac, spec.u0.T.ravel(), 0.0, O.fixed_rows(spec.tri, osys.conds), callback=cb)
    ref = ref.reshape(-1, N).T
    alg = F.NewtonRaphson() if method == "newton" else F.DynamicSS(F.TRBDF2(), abstol=1e-10, reltol=1e-10)
    sol = F.solve(F.SteadyFVMProblem(sys_), alg)
    assert sol.u.shape == (N, spec.tri.num_points)
    assert np.max(np.abs(sol.u - ref)) <= 1e-8 * np.max(np.abs(ref))
    assert np.max(np.abs(ref[0] - 1.0)) > 1e-2  # the steady state is not the boundary values
    if method == "newton":
        assert abs(sol.stats["iterations"] - it) <= 1
