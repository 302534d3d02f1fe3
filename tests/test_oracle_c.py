"""The C restatement used as the timed CPU baseline agrees with the numpy oracle
(serial and threaded, the latter mirroring parallel_fvm_eqs!)."""
import numpy as np

import build_oracle as B
import fvm_oracle as O
from problems import oracle_problem, readme_diffusion, sine_diffusion


def _cproblem(spec, kind, param):
    prob = oracle_problem(spec)
    return prob, B.CProblem(prob.geo, spec.tri, prob.code, kind, param, prob.bnd_tri)


def test_c_oracle_matches_numpy_oracle():
    for spec, kind, param in ((readme_diffusion(50), B.D_CONST, (1 / 9,)), (sine_diffusion(40), B.D_SINE, (0.5,))):
        prob, cp = _cproblem(spec, kind, param)
        u = spec.u0 + np.random.default_rng(0).random(spec.tri.num_points)
        ref = O.fvm_eqs(prob, u, 0.0)
        for got in (cp.rhs_serial(u), cp.rhs_threaded(u, nthreads=3), cp.rhs_threaded(u, nthreads=1)):
            assert np.linalg.norm(got - ref) <= 1e-13 * np.linalg.norm(ref)


def test_c_gray_scott_system_matches_numpy_oracle():
    """The C restatement of the Gray-Scott FVMSystem (the system row's CPU baseline) agrees with
    the oracle's system_fvm_eqs."""
    from fvmgpu.meshes import triangulate_rectangle

    tri = triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, 30, 30, single_boundary=True)
    bc = lambda x, y, t, u: 0.0 * x  # noqa: E731
    conds = [O.Conditions(tri, [bc], ["Neumann"]) for _ in range(2)]
    fluxes = [lambda x, y, t, a, b, g: (-a[0] * 2e-5, -b[0] * 2e-5), lambda x, y, t, a, b, g: (-a[1] * 1e-5, -b[1] * 1e-5)]
    sources = [lambda x, y, t, u: 0.04 * (1 - u[0]) - u[0] * u[1] ** 2, lambda x, y, t, u: -0.1 * u[1] + u[0] * u[1] ** 2]
    sys_ = O.System(tri, conds, fluxes, sources)
    u = np.random.default_rng(1).random((2, tri.num_points))
    ref = O.system_fvm_eqs(sys_, u, 0.0)
    cp = B.CGrayScott(sys_.geo, tri, sys_.code[0], sys_.bnd_tri)
    for nth in (1, 3):
        got = cp.rhs_threaded(u, nthreads=nth)
        for c in range(2):
            assert np.max(np.abs(got[c] - ref[c])) <= 1e-13 * np.max(np.abs(ref[c]))


def test_threaded_steady_bicgstab_matches_direct_solve():
    """The CPU baseline of the steady templates (threaded Jacobi BiCGStab in C) reaches the
    requested residual and the direct solution on a disk Poisson problem with the D jump."""
    import build_oracle as B
    from fvmgpu.meshes import triangulate_disk

    tri = triangulate_disk(3000, 128, seed=2)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_poisson(tri, conds, lambda x, y: np.where(x * x + y * y < 0.25, 1.0, 10.0),
                              lambda x, y: -1.0 + 0.0 * x)
    ref = O.steady_solve(A, b)
    V = O.Geometry(tri.points, tri.triangles).cv_volumes
    for v in (None, V):  # A x = b directly, and the GPU solver's reduced system
        x, st = B.steady_bicgstab(A, b, rtol=1e-10, nthreads=2, V=v)
        assert st["converged"] and st["rel_residual"] <= 1e-10
        assert np.linalg.norm(b - A @ x) <= 1.5e-10 * np.linalg.norm(b)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref)
        x2, st2 = B.steady_bicgstab(A, b, rtol=1e-10, nthreads=2, V=v)
        assert np.array_equal(x, x2) and st2["iterations"] == st["iterations"]  # fixed summation order
