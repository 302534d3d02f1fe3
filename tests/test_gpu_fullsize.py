"""GPU parity at the sizes the benchmark measures, against the oracle.

- 1000 x 1000 diffusion (1M vertices, the headline RHS): fvm_eqs! through the C ABI on every
  kernel path (streamed operator, difference form, per-triangle kernel, FP32 assembly) against
  the numpy oracle and the C restatement of parallel_fvm_eqs!;
- the same mesh as a DiffusionEquation: A (values and pattern), b and the A u + b product
  against the oracle's sparse assembly;
- the 500k-point disk Poisson problem (D = 1 / 10 jump): A and b against the oracle;
- the 256-instance batch on 256 x 256: FP32 batched RHS of spot-checked instances against the
  FP64 oracle RHS.

Tolerances are those of the small-mesh tests: ||du - ref|| <= tol (||ref|| + ||scale||) with
scale the per-vertex sum of term magnitudes, tol = 1e-12 in FP64 and 2e-5 in FP32 (normwise and
max-norm); template entries within 1e-12 of the largest entry.
"""
import numpy as np
import pytest

import fvm_oracle as O
from problems import api_problem, c2_diffusion, fourier_logfield, oracle_problem, parity_error, rhs_term_scale

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
FP32_RTOL = 2e-5


def _errs(got, ref, scale):
    e2 = parity_error(got, ref, scale)
    einf = np.max(np.abs(got - ref)) / np.max(np.abs(ref) + scale)
    return e2, einf


@pytest.fixture(scope="module")
def c2():
    spec = c2_diffusion(1000)
    oprob = oracle_problem(spec)
    rng = np.random.default_rng(2024)
    fields = {"gaussian": spec.u0.copy(), "rough": spec.u0 + 0.1 * rng.standard_normal(spec.tri.num_points)}
    refs = {k: (O.fvm_eqs(oprob, u, 0.0), rhs_term_scale(oprob, u, 0.0)) for k, u in fields.items()}
    return spec, oprob, fields, refs


def test_c2_rhs_every_path_against_oracle(gpu_lib, c2):
    import fvmgpu as F

    spec, oprob, fields, refs = c2
    prob = api_problem(spec)
    for name, u in fields.items():
        ref, scale = refs[name]
        for force, cons in ((False, False), (False, True), (True, False)):
            du = F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0, force_triangle=force, conservative=cons)
            e2, einf = _errs(du, ref, scale)
            assert e2 <= FP64_RTOL and einf <= FP64_RTOL, (name, force, cons, e2, einf)


def test_c2_rhs_page_locked_host_arrays_against_oracle(gpu_lib, c2):
    """The headline's end-to-end call: page-locked host u and du take the one-launch path that
    overlaps the link transfers with the product.  Against the oracle at 1e-12, and bit-identical
    to the device-array path, over repeated calls."""
    import torch

    import fvmgpu as F

    spec, oprob, fields, refs = c2
    prob = api_problem(spec)
    n = spec.tri.num_points
    u_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    du_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    for name, u in fields.items():
        ref, scale = refs[name]
        u_pin.numpy()[:] = u
        dev = F.fvm_eqs(torch.zeros(n, dtype=torch.float64, device="cuda"), u_pin.cuda(), prob, 0.0).cpu().numpy()
        for _ in range(3):
            du_pin.numpy()[:] = np.nan
            F.fvm_eqs(du_pin.numpy(), u_pin.numpy(), prob, 0.0)
            assert np.array_equal(du_pin.numpy(), dev), name
        e2, einf = _errs(du_pin.numpy(), ref, scale)
        assert e2 <= FP64_RTOL and einf <= FP64_RTOL, (name, e2, einf)


def test_c2_rhs_fp32_against_oracle(gpu_lib, c2):
    import fvmgpu as F

    spec, oprob, fields, refs = c2
    prob = api_problem(spec, precision="fp32")
    for name, u in fields.items():
        ref, scale = refs[name]
        for cons in (False, True):
            du = F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0, conservative=cons)
            e2, _ = _errs(du, ref, scale)
            assert e2 <= FP32_RTOL, (name, cons, e2)


def test_c2_rhs_against_c_restatement(gpu_lib, c2):
    """The C restatement of parallel_fvm_eqs! (the CPU baseline) on the same 1M-vertex inputs."""
    import build_oracle as B
    import fvmgpu as F

    spec, oprob, fields, refs = c2
    cp = B.CProblem(oprob.geo, spec.tri, oprob.code, B.D_SINE, (0.5,), oprob.bnd_tri)
    prob = api_problem(spec)
    for name, u in fields.items():
        ref_c = cp.rhs_threaded(u)
        _, scale = refs[name]
        du = F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0)
        e2, einf = _errs(du, ref_c, scale)
        assert e2 <= FP64_RTOL and einf <= FP64_RTOL, (name, e2, einf)


def test_c2_connectivity_bit_exact(gpu_lib, c2):
    spec, oprob, _, _ = c2
    prob = api_problem(spec)
    tris, belems = prob.mesh.export_connectivity()
    assert np.array_equal(tris, spec.tri.triangles)
    assert np.array_equal(belems[:, :2], spec.tri.boundary_edges)
    assert np.array_equal(belems[:, 2], spec.tri.boundary_adjacent)
    code, _ = prob.export_codes()
    assert np.array_equal(code, oprob.code)


def _assert_same_operator(A_gpu, A_ref, tol=1e-12):
    """Values within tol of the largest entry, and the same pattern of entries that are not
    rounding-level (|a| > tol max|A|): the reference's dense-then-sparse assembly keeps an entry
    exactly when its accumulated value is non-zero, so entries that cancel to a few ulps of the
    largest entry may be stored on one side only."""
    A_gpu, A_ref = A_gpu.tocsr(), A_ref.tocsr()
    big = abs(A_ref).max()
    assert abs(A_gpu - A_ref).max() <= tol * big
    g, r = A_gpu.copy(), A_ref.copy()
    g.data[np.abs(g.data) <= tol * big] = 0.0
    r.data[np.abs(r.data) <= tol * big] = 0.0
    g.eliminate_zeros()
    r.eliminate_zeros()
    g.sort_indices()
    r.sort_indices()
    assert np.array_equal(g.indptr, r.indptr) and np.array_equal(g.indices, r.indices)


def test_c2_diffusion_template_against_oracle(gpu_lib, c2):
    import fvmgpu as F

    spec, _, fields, _ = c2
    mesh = F.FVMGeometry(spec.tri)
    BCs = F.BoundaryConditions(mesh, spec.bc_fns, (F.Dirichlet,) * 4)
    D = lambda x, y, p: spec.D(x, y, 0.0, 0.0, None)  # noqa: E731
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=D, initial_condition=spec.u0, final_time=1e-4)
    conds = O.Conditions(spec.tri, [lambda x, y, t, u: 0.0 * x] * 4, ["Dirichlet"] * 4)
    A, b, u0 = O.template_diffusion(spec.tri, conds, lambda x, y: D(x, y, None), spec.u0)
    _assert_same_operator(tmpl.A, A)
    assert np.array_equal(tmpl.b, b) and np.array_equal(tmpl.u0, u0)
    u = fields["rough"]
    ref = A @ u + b
    for prec, tol in (("fp64", FP64_RTOL), ("fp32", FP32_RTOL)):
        du = tmpl.apply(np.zeros_like(u), u, precision=prec)
        scale = abs(A) @ np.abs(u) + np.abs(b)
        e2, einf = _errs(du, ref, scale)
        assert e2 <= tol and (prec == "fp32" or einf <= tol), (prec, e2, einf)


def test_c3_poisson_operator_500k_against_oracle(gpu_lib):
    """The disk Poisson workload at 500,000 interior points + 4096 boundary points: the GPU's
    assembled A and b against the oracle's PoissonsEquation assembly."""
    import fvmgpu as F

    tri = F.triangulate_disk(500_000, 4096, seed=0)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, lambda x, y, t, u, p: 0.0 * x, F.Dirichlet)
    D = lambda x, y, p: np.where(x * x + y * y < 0.25, 1.0, 10.0)  # noqa: E731
    pois = F.PoissonsEquation(mesh, BCs, diffusion_function=D, source_function=lambda x, y, p: -1.0 + 0.0 * x)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_poisson(tri, conds, lambda x, y: D(x, y, None), lambda x, y: -1.0 + 0.0 * x)
    _assert_same_operator(pois.A, A)
    assert np.array_equal(pois.b, b)


def test_c4_fp32_batch_against_fp64_oracle(gpu_lib):
    """256 instances on 256 x 256 (log-normal D per instance, sigma = 0.5, 16 Fourier modes,
    linear reaction f = -1, zero Dirichlet), FP32 state and arithmetic: instances spread over
    the batch against the FP64 oracle RHS of the same (FP32-rounded) state."""
    import fvmgpu as F
    from fvmgpu.meshes import triangulate_rectangle

    B = 256
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 256, 256, single_boundary=True)
    mesh = F.FVMGeometry(tri)
    BCs = F.BoundaryConditions(mesh, lambda x, y, t, u, p: 0.0 * x, F.Dirichlet)
    P = tri.points
    u0 = np.exp(-50 * ((P[:, 0] - 0.5) ** 2 + (P[:, 1] - 0.5) ** 2))
    react = lambda x, y, t, u, p: -1.0 * u  # noqa: E731
    prob = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x, source_function=react,
                        initial_condition=u0, final_time=1e-4)
    logDs = [fourier_logfield(seed) for seed in range(B)]
    dual, quarter = mesh.sample_points()
    Ps = np.vstack([dual.reshape(-1, 2), quarter.reshape(-1, 2)])
    Dall = np.stack([np.exp(f(Ps[:, 0], Ps[:, 1])) for f in logDs])
    b32 = F.BatchedProblem(prob, Dall, precision="fp32")
    n = tri.num_points
    U = np.ascontiguousarray(np.random.default_rng(5).random((n, B)), dtype=np.float32)
    dU = b32.rhs(np.zeros((n, B), dtype=np.float32), U)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    for b in (0, 37, 128, 255):
        f = logDs[b]
        op = O.Problem(tri, conds, D=lambda x, y, t, u, f=f: np.exp(f(x, y)) + 0.0 * u,
                       source=lambda x, y, t, u: -1.0 * u, u0=u0)
        u = U[:, b].astype(np.float64)
        ref = O.fvm_eqs(op, u, 0.0)
        scale = rhs_term_scale(op, u, 0.0)
        e2, _ = _errs(dU[:, b].astype(np.float64), ref, scale)
        assert e2 <= FP32_RTOL, (b, e2)
