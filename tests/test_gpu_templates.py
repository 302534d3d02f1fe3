"""Linear templates on the GPU against the oracle's sparse restatement: the assembled A and b
(max-norm 1e-12 relative), the A u + b operator (FP64 1e-12, FP32 2e-5) and the steady
solves (FP64 Krylov, mixed precision, BiCGStab) to ||b - A x|| / ||b|| <= 1e-10."""
import numpy as np
import pytest

import fvm_oracle as O
from problems import sine_diffusion
from fvmgpu.meshes import triangulate_disk, triangulate_rectangle

pytestmark = pytest.mark.gpu


def _maxrel(A, B):
    d = (A - B)
    d = abs(d).max() if hasattr(d, "nnz") else np.max(np.abs(d))
    s = abs(B).max() if hasattr(B, "nnz") else np.max(np.abs(B))
    return d / max(s, 1e-300)


def _mesh_bcs(F, tri, fns, types):
    mesh = F.FVMGeometry(tri)
    return mesh, F.BoundaryConditions(mesh, tuple(fns), tuple(getattr(F, t) for t in types))


def test_diffusion_template_assembly_and_apply(gpu_lib):
    import fvmgpu as F

    spec = sine_diffusion(48)
    mesh, BCs = _mesh_bcs(F, spec.tri, [spec.bc_fns[0]], ["Dirichlet"])
    D = lambda x, y, p: spec.D(x, y, 0, 0, None)  # noqa: E731
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=D, initial_condition=spec.u0, final_time=1.0)
    conds = O.Conditions(spec.tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b, u0 = O.template_diffusion(spec.tri, conds, lambda x, y: D(x, y, None), spec.u0)
    assert _maxrel(tmpl.A, A) < 1e-12
    assert np.allclose(tmpl.b, b) and np.allclose(tmpl.u0, u0)
    u = np.random.default_rng(0).random(spec.tri.num_points)
    for prec, tol in (("fp64", 1e-12), ("fp32", 2e-5)):
        du = tmpl.apply(np.zeros_like(u), u, precision=prec)
        ref = A @ u + b
        assert np.linalg.norm(du - ref) / np.linalg.norm(ref) < tol


def test_neumann_template_quirk_and_lrd(gpu_lib):
    """Boundary rows of a Neumann / non-Neumann mixture (abstract_templates.jl:175-191 and the
    V_i division of row j at :262) and the linear reaction term (:115-125)."""
    import fvmgpu as F

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 2.0, 17, 23, single_boundary=False)
    fns = [lambda x, y, t, u, p: 0.5 + 0.0 * x, lambda x, y, t, u, p: x * 0.0 + 1.0,
           lambda x, y, t, u, p: y * 0.1, lambda x, y, t, u, p: 0.0 * x]
    types = ["Neumann", "Dirichlet", "Neumann", "Constrained"]
    mesh, BCs = _mesh_bcs(F, tri, fns, types)
    D = lambda x, y, p: 1.0 + x * y  # noqa: E731
    f = lambda x, y, p: -0.3 + 0.1 * x  # noqa: E731
    u0 = np.random.default_rng(1).random(tri.num_points)
    lrd = F.LinearReactionDiffusionEquation(mesh, BCs, diffusion_function=D, source_function=f, initial_condition=u0,
                                            final_time=1.0)
    conds = O.Conditions(tri, [lambda x, y, t, u, g=g: g(x, y, t, u, None) for g in fns], types)
    A, b, _ = O.template_diffusion(tri, conds, lambda x, y: D(x, y, None), u0, reaction=lambda x, y: f(x, y, None))
    assert _maxrel(lrd.A, A) < 1e-12
    assert np.max(np.abs(lrd.b - b)) <= 1e-12 * max(1.0, np.max(np.abs(b)))


def test_poisson_exact_solution_gpu(gpu_lib):
    """docs/src/literate_wyos/poissons_equation.jl:92-116: u = sin(pi x) sin(pi y)/(2 pi^2)."""
    import fvmgpu as F

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 100, 100, single_boundary=True)
    mesh, BCs = _mesh_bcs(F, tri, [lambda x, y, t, u, p: 0.0 * x], ["Dirichlet"])
    prob = F.PoissonsEquation(mesh, BCs, source_function=lambda x, y, p: -np.sin(np.pi * x) * np.sin(np.pi * y))
    P = tri.points
    exact = np.sin(np.pi * P[:, 0]) * np.sin(np.pi * P[:, 1]) / (2 * np.pi**2)
    for mode, precond in (("fp64", "jacobi"), ("mixed", "jacobi"), ("fp64", "chebyshev"), ("mixed", "chebyshev")):
        sol = F.solve(prob, F.KrylovSolver(mode=mode, precond=precond))
        assert sol.stats["rel_residual"] <= 1e-10
        assert np.linalg.norm(sol.u - exact) <= 1e-4 * np.linalg.norm(exact)


def test_laplace_template_is_poisson_without_a_source(gpu_lib):
    """LaplacesEquation (laplaces_equation.jl:48-94) assembles as the Poisson template with f = 0:
    its solution equals PoissonsEquation's with a zero source bit for bit, and with the boundary
    values 0, 100y, 100, 100y it is u = 100y, which the scheme reproduces."""
    import fvmgpu as F

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 40, 40, single_boundary=False)
    fns = [lambda x, y, t, u, p: 0.0 * x, lambda x, y, t, u, p: 100 * y, lambda x, y, t, u, p: 100.0 + 0.0 * x,
           lambda x, y, t, u, p: 100 * y]
    mesh, BCs = _mesh_bcs(F, tri, fns, ["Dirichlet"] * 4)
    lap = F.solve(F.LaplacesEquation(mesh, BCs))
    pois = F.solve(F.PoissonsEquation(mesh, BCs, source_function=lambda x, y, p: 0.0 * x))
    assert np.array_equal(lap.u, pois.u)
    assert np.max(np.abs(lap.u - 100 * tri.points[:, 1])) <= 1e-6 * 100


@pytest.mark.parametrize("precond", ["jacobi", "chebyshev"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("jump", [False, True])
def test_steady_disk_against_direct_solve(gpu_lib, mode, jump, precond):
    """Disk Poisson (f = -1) with D = 1 or the 1 / 10 jump at r = 0.5 (non-symmetric operator:
    BiCGStab), Jacobi or Chebyshev (degree 4) preconditioning, against scipy's direct solve of
    the oracle's assembled system."""
    import fvmgpu as F

    tri = triangulate_disk(6000, 256, seed=4)
    mesh, BCs = _mesh_bcs(F, tri, [lambda x, y, t, u, p: 0.0 * x], ["Dirichlet"])
    D = (lambda x, y, p: np.where(x * x + y * y < 0.25, 1.0, 10.0)) if jump else (lambda x, y, p: 1.0 + 0.0 * x)
    prob = F.PoissonsEquation(mesh, BCs, diffusion_function=D, source_function=lambda x, y, p: -1.0 + 0.0 * x)
    sol = F.solve(prob, F.KrylovSolver(mode=mode, rtol=1e-10, precond=precond))
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_poisson(tri, conds, lambda x, y: D(x, y, None), lambda x, y: -1.0 + 0.0 * x)
    ref = O.steady_solve(A, b)
    res = np.linalg.norm(b - A @ sol.u) / np.linalg.norm(b)
    assert res <= 1e-10, (res, sol.stats)
    assert np.linalg.norm(sol.u - ref) <= 1e-7 * np.linalg.norm(ref)
    assert sol.stats["method"] == ("bicgstab" if jump else "cg")
    if precond == "chebyshev":  # fewer outer iterations than Jacobi alone
        jac = F.solve(prob, F.KrylovSolver(mode=mode, rtol=1e-10))
        assert sol.stats["iterations"] < jac.stats["iterations"], (sol.stats, jac.stats)


@pytest.mark.parametrize("jump", [False, True])
def test_steady_fp32_stored_preconditioner(gpu_lib, jump):
    """FP64 Krylov with a Chebyshev preconditioner on FP32-stored operator values (FP64
    vectors and arithmetic, so a fixed linear preconditioner): the same 1e-10 FP64 residual
    without falling back, and about as many iterations as the all-FP64 solve."""
    import fvmgpu as F

    tri = triangulate_disk(6000, 256, seed=4)
    mesh, BCs = _mesh_bcs(F, tri, [lambda x, y, t, u, p: 0.0 * x], ["Dirichlet"])
    D = (lambda x, y, p: np.where(x * x + y * y < 0.25, 1.0, 10.0)) if jump else (lambda x, y, p: 1.0 + 0.0 * x)
    prob = F.PoissonsEquation(mesh, BCs, diffusion_function=D, source_function=lambda x, y, p: -1.0 + 0.0 * x)
    sol = F.solve(prob, F.KrylovSolver(mode="fp32_precond", precond="chebyshev", rtol=1e-10))
    ref64 = F.solve(prob, F.KrylovSolver(mode="fp64", precond="chebyshev", rtol=1e-10))
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_poisson(tri, conds, lambda x, y: D(x, y, None), lambda x, y: -1.0 + 0.0 * x)
    assert np.linalg.norm(b - A @ sol.u) / np.linalg.norm(b) <= 1e-10
    assert np.linalg.norm(sol.u - O.steady_solve(A, b)) <= 1e-7 * np.linalg.norm(sol.u)
    assert not sol.stats["fallback_fp64"]
    assert sol.stats["iterations"] <= 1.5 * ref64.stats["iterations"] + 16, (sol.stats, ref64.stats)
    with pytest.raises(F.FVMError):  # the FP32-stored operator is the Chebyshev preconditioner's
        F.solve(prob, F.KrylovSolver(mode="fp32_precond", precond="jacobi"))


def test_mean_exit_time_gpu(gpu_lib):
    import fvmgpu as F

    tri = triangulate_disk(5000, 200, seed=5)
    mesh, BCs = _mesh_bcs(F, tri, [lambda x, y, t, u, p: 0.0 * x], ["Dirichlet"])
    met = F.MeanExitTimeProblem(mesh, BCs, diffusion_function=lambda x, y, p: 1.0 + 0.0 * x)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_mean_exit_time(tri, conds, lambda x, y: 1.0 + 0.0 * x)
    assert _maxrel(met.A, A) < 1e-12
    sol = F.solve(met, F.KrylovSolver(mode="mixed"))
    assert np.linalg.norm(b - A @ sol.u) / np.linalg.norm(b) <= 1e-10


def test_template_argument_errors(gpu_lib):
    """poissons_equation.jl:69-70 and mean_exit_time.jl:66-69 raise ArgumentError."""
    import fvmgpu as F

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 8, 8, single_boundary=False)
    mesh = F.FVMGeometry(tri)
    z = lambda x, y, t, u, p: 0.0 * x  # noqa: E731
    BCs = F.BoundaryConditions(mesh, (z,) * 4, (F.Dirichlet, F.Dudt, F.Dirichlet, F.Dirichlet))
    with pytest.raises(ValueError, match="Dudt"):
        F.PoissonsEquation(mesh, BCs, source_function=lambda x, y, p: 0.0 * x)
    BCs = F.BoundaryConditions(mesh, (z,) * 4, (F.Dirichlet, F.Constrained, F.Dirichlet, F.Dirichlet))
    with pytest.raises(ValueError, match="Constrained"):
        F.MeanExitTimeProblem(mesh, BCs, diffusion_function=lambda x, y, p: 1.0 + 0.0 * x)
