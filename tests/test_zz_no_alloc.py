"""fvm_rhs_noalloc: the RHS entry point for callers that cannot allocate device memory.

Such callers include real-time loops with a frozen allocator and hosts that give all device
memory to their own pool, where a cudaMalloc behind the pool's back fails or fragments it.  The test calls the
entry point through the C ABI, twice in a row with different inputs, and checks each result
against the allocating entry point fvm_rhs.  It uses the same FP64 tolerance as the other RHS
tests (1e-12 relative); both paths run the same kernels, so the results are identical.  The
second call shows that scratch left over from the first call does not leak into it.  The
file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from problems import api_problem, mixed_annulus, nonlinear_rect, readme_diffusion

pytestmark = pytest.mark.gpu


def _rhs(lib, prob, u, noalloc):
    import torch

    du = torch.full_like(u, float("nan"))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if noalloc:
        st = lib.fvm_rhs_noalloc(prob.handle, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(du.data_ptr()), 0.0,
                                 stream)
    else:
        st = lib.fvm_rhs(prob.handle, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(du.data_ptr()), 0.0, 1, stream)
    torch.cuda.synchronize()
    return st, du.cpu().numpy()


@pytest.mark.parametrize("builder", [lambda: readme_diffusion(50), mixed_annulus, lambda: nonlinear_rect(30)],
                         ids=["readme50", "mixed_annulus", "nonlinear30"])
def test_noalloc_matches_allocating_entry_point(gpu_lib, builder):
    import torch

    lib = gpu_lib.load()
    spec = builder()
    prob = api_problem(spec)
    rng = np.random.default_rng(21)
    for call in range(2):
        u = torch.tensor(spec.u0 + 0.1 * rng.standard_normal(spec.tri.num_points), device="cuda")
        st_ref, ref = _rhs(lib, prob, u, noalloc=False)
        assert st_ref == 0, gpu_lib.last_error()
        st, got = _rhs(lib, prob, u, noalloc=True)
        assert st == 0, gpu_lib.last_error()
        assert np.all(np.isfinite(got))
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), call


def test_noalloc_rejects_meshes_above_the_limit(gpu_lib):
    import torch
    import fvmgpu as F

    lib = gpu_lib.load()
    n = 520  # 520 x 520 = 270,400 points > FVM_NOALLOC_MAX_POINTS = 262,144
    tri = F.triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, lambda x, y, t, u, p: 0.0 * x, F.Dirichlet)
    prob = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                        initial_condition=np.zeros(tri.num_points), final_time=1.0)
    u = torch.zeros(tri.num_points, dtype=torch.float64, device="cuda")
    du = torch.zeros_like(u)
    st = lib.fvm_rhs_noalloc(prob.handle, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(du.data_ptr()), 0.0, None)
    assert st == gpu_lib.FVM_ERR_INVALID_ARGUMENT
    assert "262144" in gpu_lib.last_error()


def test_noalloc_refuses_a_fresh_nonlinear_problem(gpu_lib):
    """A nonlinear problem's per-triangle data is built by its first fvm_rhs call; before that
    the no-allocation entry point refuses it (it never allocates lazily), and after one
    fvm_rhs call it runs."""
    import torch

    lib = gpu_lib.load()
    spec = nonlinear_rect(20)
    prob = api_problem(spec)
    u = torch.tensor(spec.u0, device="cuda")
    st, _ = _rhs(lib, prob, u, noalloc=True)
    assert st == gpu_lib.FVM_ERR_INVALID_ARGUMENT
    assert "fvm_rhs" in gpu_lib.last_error()
    st_ref, ref = _rhs(lib, prob, u, noalloc=False)
    assert st_ref == 0, gpu_lib.last_error()
    st, got = _rhs(lib, prob, u, noalloc=True)
    assert st == 0, gpu_lib.last_error()
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
