"""Batched instances and the multi-mesh batch against per-instance GPU problems (which are
themselves checked against the oracle).  FP64 batch within 1e-12 relative of the
per-instance RHS, FP32 batch within 2e-5; batched Tsit5 within 1e-10 (FP64) / 1e-4 (FP32)."""
import numpy as np
import pytest

from problems import api_problem, oracle_problem, sine_diffusion
import fvm_oracle as O

pytestmark = pytest.mark.gpu


def lognormal_fields(B, seed=0, sigma=0.5, modes=16):
    """log D = sigma sum_m a_m cos(2 pi k_m . x + phi_m) / sqrt(modes / 2), seeded."""
    rng = np.random.default_rng(seed)
    fields = []
    for _ in range(B):
        a = rng.standard_normal(modes)
        k = rng.integers(1, 5, size=(modes, 2))
        ph = rng.uniform(0, 2 * np.pi, modes)

        def D(x, y, t, u, p, a=a, k=k, ph=ph):
            s = sum(a[m] * np.cos(2 * np.pi * (k[m, 0] * x + k[m, 1] * y) + ph[m]) for m in range(modes))
            return np.exp(sigma * s / np.sqrt(modes / 2)) + 0.0 * u
        fields.append(D)
    return fields


def _base(n=40):
    spec = sine_diffusion(n)
    spec.S = lambda x, y, t, u, p: -1.0 * u  # linear reaction f = -1 (LinearReactionDiffusionEquation form)
    return spec


@pytest.mark.parametrize("B", [1, 8, 64])
def test_batched_rhs_matches_instances(gpu_lib, B):
    import fvmgpu as F

    spec = _base()
    Ds = lognormal_fields(B, seed=B)
    prob = api_problem(spec)
    batch = F.BatchedProblem(prob, Ds)
    n = spec.tri.num_points
    rng = np.random.default_rng(1)
    U = np.ascontiguousarray(rng.random((n, B)))
    dU = batch.rhs(np.zeros((n, B)), U)
    for b in range(0, B, max(1, B // 4)):
        spec.D = Ds[b]
        pb = api_problem(spec, mesh=prob.mesh)
        ref = F.fvm_eqs(np.zeros(n), np.ascontiguousarray(U[:, b]), pb, 0.0)
        assert np.linalg.norm(dU[:, b] - ref) <= 1e-12 * np.linalg.norm(ref), b
    t = batch.tuning()
    assert t["block"] in (128, 256, 512) and t["instances_per_thread"] in (1, 2) and t["grid"] > 0


def test_batched_rhs_against_oracle_and_fp32(gpu_lib):
    import fvmgpu as F

    spec = _base(24)
    Ds = lognormal_fields(4, seed=7)
    prob = api_problem(spec)
    b64 = F.BatchedProblem(prob, Ds)
    b32 = F.BatchedProblem(prob, Ds, precision="fp32")
    n = spec.tri.num_points
    U = np.random.default_rng(2).random((n, 4))
    d64 = b64.rhs(np.zeros((n, 4)), np.ascontiguousarray(U))
    d32 = b32.rhs(np.zeros((n, 4), dtype=np.float32), np.ascontiguousarray(U, dtype=np.float32))
    assert b32.tuning()["instances_per_thread"] in (1, 2, 4)
    for b in range(4):
        spec.D = Ds[b]
        ref = O.fvm_eqs(oracle_problem(spec), U[:, b], 0.0)
        assert np.linalg.norm(d64[:, b] - ref) <= 1e-12 * np.linalg.norm(ref)
        assert np.linalg.norm(d32[:, b] - ref) <= 2e-5 * np.linalg.norm(ref)


def test_batched_tsit5_matches_instances(gpu_lib):
    import fvmgpu as F

    spec = _base(32)
    spec.tf = 2e-3
    Ds = lognormal_fields(8, seed=3)
    prob = api_problem(spec)
    batch = F.BatchedProblem(prob, Ds)
    ts, out, st = batch.solve(spec.u0, dt=1e-4, saveat=[1e-3, 2e-3])
    assert st["steps"] == 20 and out.shape == (2, spec.tri.num_points, 8)
    b32 = F.BatchedProblem(prob, Ds, precision="fp32")
    _, out32, _ = b32.solve(spec.u0, dt=1e-4, saveat=[1e-3, 2e-3])
    for b in (0, 5):
        spec.D = Ds[b]
        pb = api_problem(spec, mesh=prob.mesh)
        sol = F.solve(pb, F.Tsit5(), dt=1e-4, adaptive=False, saveat=[1e-3, 2e-3])
        for k in range(2):
            ref = sol.u[k]
            assert np.max(np.abs(out[k, :, b] - ref)) <= 1e-10 * np.max(np.abs(ref))
            assert np.max(np.abs(out32[k, :, b] - ref)) <= 1e-4 * np.max(np.abs(ref))


def test_multimesh_union_steps_every_mesh(gpu_lib):
    """Meshes of uneven sizes in one problem: one launch per RHS, one graph per step."""
    import fvmgpu as F

    sizes = (12, 31, 20)
    tris = [F.triangulate_rectangle(0.0, 1.0, 0.0, 1.0, s, s, single_boundary=True) for s in sizes]
    U, poff, soff = F.disjoint_union(tris)
    D = lambda x, y, t, u, p: 1.0 + 0.3 * x + 0.0 * u  # noqa: E731
    z = lambda x, y, t, u, p: 0.0 * x  # noqa: E731
    u0 = np.exp(-20 * ((U.points[:, 0] - 0.5) ** 2 + (U.points[:, 1] - 0.5) ** 2))
    mesh = F.FVMGeometry(U)
    BCs = F.BoundaryConditions(mesh, (z,) * U.num_ghost_vertices, (F.Dirichlet,) * U.num_ghost_vertices)
    prob = F.FVMProblem(mesh, BCs, diffusion_function=D, initial_condition=u0, final_time=1e-3)
    sol = F.solve(prob, F.Tsit5(), dt=1e-4, adaptive=False, saveat=[1e-3])
    for m, t in enumerate(tris):
        mm = F.FVMGeometry(t)
        pm = F.FVMProblem(mm, F.BoundaryConditions(mm, z, F.Dirichlet), diffusion_function=D,
                          initial_condition=u0[poff[m]:poff[m + 1]], final_time=1e-3)
        sm = F.solve(pm, F.Tsit5(), dt=1e-4, adaptive=False, saveat=[1e-3])
        got = sol.u[-1][poff[m]:poff[m + 1]]
        assert np.max(np.abs(got - sm.u[-1])) <= 1e-12 * np.max(np.abs(sm.u[-1]))
