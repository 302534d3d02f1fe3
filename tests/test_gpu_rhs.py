"""GPU parity of fvm_eqs! (libfvmgpu through the C ABI) against the oracle.

Tolerances, relative to the size of what is summed: ||du - ref|| <= tol (||ref|| + ||scale||),
where scale is the per-vertex sum of term magnitudes (problems.rhs_term_scale) - any
floating-point evaluation, the reference's included, is defined only to ~eps times it.
FP64: tol = 1e-12 (normwise and max-norm); FP32 assembly: tol = 2e-5.  Integer tables
(connectivity, classification) bit-exact.
"""
import numpy as np
import pytest

import fvm_oracle as O
from problems import (api_problem, heat_convection, mixed_annulus, nonlinear_rect, oracle_problem, parity_error,
                      readme_diffusion, rhs_term_scale, sine_diffusion, wheel_diffusion)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
FP32_RTOL = 2e-5


def rel_err(got, ref, scale=None):
    """(normwise, max-norm) error relative to |ref| + scale."""
    sc = np.zeros_like(ref) if scale is None else scale
    e2 = parity_error(got, ref, sc)
    einf = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref) + sc), 1e-300)
    return e2, einf


BUILDERS = {
    "readme50": lambda: readme_diffusion(50),
    "heat_convection200": lambda: heat_convection(200),
    "mixed_annulus": mixed_annulus,
    "sine64": lambda: sine_diffusion(64),
    "nonlinear30": lambda: nonlinear_rect(30),
    "wheel40": lambda: wheel_diffusion(40),  # slices wider than 16 slots: the one-warp-per-slice kernel
}


@pytest.mark.parametrize("name", list(BUILDERS))
def test_rhs_parity_fp64(gpu_lib, name):
    import fvmgpu as F

    spec = BUILDERS[name]()
    oprob = oracle_problem(spec)
    rng = np.random.default_rng(11)
    P = spec.tri.points
    # a smooth field on the problem's own offset, and a rough one
    for trial in range(2):
        if trial == 0:
            u = spec.u0 + 0.05 * np.sin(3 * P[:, 0] + 2 * P[:, 1])
        else:
            u = spec.u0 + rng.standard_normal(spec.tri.num_points) * 0.1
        ref = O.fvm_eqs(oprob, u, spec.t0)
        scale = rhs_term_scale(oprob, u, spec.t0)
        prob = api_problem(spec)
        for force, cons in ((False, False), (False, True), (True, False)):
            du = np.zeros_like(u)
            F.fvm_eqs(du, np.ascontiguousarray(u), prob, spec.t0, force_triangle=force, conservative=cons)
            e2, einf = rel_err(du, ref, scale)
            assert e2 <= FP64_RTOL and einf <= FP64_RTOL, (name, force, cons, e2, einf)


def test_constant_field_exact(gpu_lib):
    """test/equations.jl:37-92 on the GPU: heat convection at T = 10 everywhere.  With
    FVM_RHS_CONSERVATIVE interior fluxes vanish exactly, the corner vertex matches the
    hand-computed value, and only Neumann boundary rows are non-zero."""
    import fvmgpu as F

    spec = heat_convection(200)
    prob = api_problem(spec)
    du = F.fvm_eqs(np.zeros(spec.tri.num_points), spec.u0.copy(), prob, 0.0, conservative=True)
    P = spec.tri.points
    x1, y1 = P[1, 0], P[200, 1]
    A = 0.5 * abs((x1 / 2) * (y1 / 3) - (x1 / 3) * 0.0) + 0.5 * abs((x1 / 3) * (y1 / 2) - 0.0 * (y1 / 3))
    Pm = spec.bc_params[0]
    fl = -(1 / A) * (-Pm["alpha"] * Pm["q"] / Pm["k"] * (x1 / 2))
    assert np.isclose(du[0], fl, rtol=1e-12)
    interior = np.ones(spec.tri.num_points, bool)
    interior[np.concatenate(spec.tri.boundary_nodes)] = False
    assert np.all(du[interior] == 0.0)
    top = spec.tri.boundary_nodes[2]
    assert np.max(np.abs(du[top])) <= 1e-14 * np.max(np.abs(du))


def test_rhs_parity_device_pointers(gpu_lib):
    import torch
    import fvmgpu as F

    spec = mixed_annulus()
    oprob = oracle_problem(spec)
    prob = api_problem(spec)
    u = torch.tensor(spec.u0, dtype=torch.float64, device="cuda")
    du = torch.zeros_like(u)
    F.fvm_eqs(du, u, {"prob": prob}, 0.0)
    torch.cuda.synchronize()
    ref = O.fvm_eqs(oprob, spec.u0, 0.0)
    e2, einf = rel_err(du.cpu().numpy(), ref)
    assert e2 <= FP64_RTOL and einf <= FP64_RTOL


@pytest.mark.parametrize("name", ["readme50", "heat_convection200", "sine64", "mixed_annulus"])
def test_rhs_parity_fp32(gpu_lib, name):
    import fvmgpu as F

    spec = BUILDERS[name]()
    oprob = oracle_problem(spec)
    ref = O.fvm_eqs(oprob, spec.u0, 0.0)
    scale = rhs_term_scale(oprob, spec.u0, 0.0)
    prob = api_problem(spec, precision="fp32")
    for cons in (False, True):
        du = np.zeros_like(spec.u0)
        F.fvm_eqs(du, np.ascontiguousarray(spec.u0, dtype=np.float64), prob, 0.0, conservative=cons)
        e2, _ = rel_err(du, ref, scale)
        assert e2 <= FP32_RTOL, (cons, e2)


@pytest.mark.parametrize("tile", [64, 256, 1024])
def test_tile_sizes_agree(gpu_lib, tile):
    import fvmgpu as F

    spec = nonlinear_rect(40)
    ref = O.fvm_eqs(oracle_problem(spec), spec.u0, 0.0)
    prob = api_problem(spec, tile_vertices=tile)
    du = np.zeros_like(spec.u0)
    F.fvm_eqs(du, spec.u0.copy(), prob, 0.0)
    e2, einf = rel_err(du, ref)
    assert e2 <= FP64_RTOL and einf <= FP64_RTOL


@pytest.mark.parametrize("name", ["mixed_annulus", "heat_convection200"])
def test_connectivity_and_classification_bit_exact(gpu_lib, name):
    """Device-resident triangles / boundary elements / vertex codes / Neumann flags, read back
    and mapped to the caller's numbering, equal the oracle's tables exactly."""
    spec = BUILDERS[name]()
    oprob = oracle_problem(spec)
    prob = api_problem(spec)
    tris, belems = prob.mesh.export_connectivity()
    assert np.array_equal(tris, spec.tri.triangles)
    assert np.array_equal(belems[:, :2], spec.tri.boundary_edges)
    assert np.array_equal(belems[:, 2], spec.tri.boundary_adjacent)
    code, neu = prob.export_codes()
    assert np.array_equal(code, oprob.code)
    assert np.array_equal(neu, (oprob.neumann_fidx >= 0).astype(np.int8))
    perm = prob.mesh.permutation()
    assert np.array_equal(np.sort(perm), np.arange(spec.tri.num_points))
    assert np.allclose(prob.mesh.cv_volumes, oprob.geo.cv_volumes, rtol=1e-14, atol=0)


def test_dirichlet_update(gpu_lib):
    import fvmgpu as F

    spec = mixed_annulus()
    oprob = oracle_problem(spec)
    prob = api_problem(spec)
    u = spec.u0.copy()
    F.update_dirichlet_nodes(u, prob, 0.0)
    ref = O.update_dirichlet_nodes(oprob, spec.u0, 0.0)
    assert np.array_equal(u, ref)


def test_unsupported_forms_are_rejected(gpu_lib):
    """Closures are classified when the problem is first used (as the reference evaluates them
    only when it solves); an unsupported one raises there, on every use.  A flux linear in
    (alpha, beta, gamma) is a device form (advection); a flux nonlinear in them is not."""
    import fvmgpu as F

    spec = readme_diffusion(10)
    spec.D = lambda x, y, t, u, p: 1.0 + np.exp(u)
    prob = api_problem(spec)
    with pytest.raises(F.UnsupportedFormError):
        prob.handle
    with pytest.raises(F.UnsupportedFormError):
        F.fvm_eqs(np.zeros_like(spec.u0), spec.u0, prob, 0.0)
    spec = readme_diffusion(10)
    spec.D = lambda x, y, t, u, p: 1.0 + t + 0.0 * x
    with pytest.raises(F.UnsupportedFormError):
        F.solve(api_problem(spec), F.Tsit5())
    spec = readme_diffusion(10)
    spec.flux = lambda x, y, t, a, b, g, p: (-a + 0.1 * g, -b)
    spec.D = None
    assert api_problem(spec).info()["linear"] == 1
    spec.flux = lambda x, y, t, a, b, g, p: (-a + 0.1 * g * g, -b)
    with pytest.raises(F.UnsupportedFormError):
        api_problem(spec).handle


def test_full_size_properties(gpu_lib):
    """1000 x 1000 (1M vertices): RHS of a constant field vanishes on free rows; linearity;
    operator path and triangle path agree."""
    import fvmgpu as F

    spec = sine_diffusion(1000)
    prob = api_problem(spec)
    n = spec.tri.num_points
    one = np.ones(n)
    du = np.zeros(n)
    F.fvm_eqs(du, one, prob, 0.0)
    code, _ = prob.export_codes()
    free = code == 0
    scale = np.max(np.abs(F.fvm_eqs(np.zeros(n), spec.u0.copy(), prob, 0.0)))
    assert np.max(np.abs(du[free])) <= 1e-12 * scale * 1e3
    rng = np.random.default_rng(12)
    u, v = rng.random(n), rng.random(n)
    a, b = 0.7, -1.3
    fu = F.fvm_eqs(np.zeros(n), u, prob, 0.0)
    fv = F.fvm_eqs(np.zeros(n), v, prob, 0.0)
    fw = F.fvm_eqs(np.zeros(n), a * u + b * v, prob, 0.0)
    e2, _ = rel_err(fw, a * fu + b * fv)
    assert e2 <= 1e-12
    ft = F.fvm_eqs(np.zeros(n), u, prob, 0.0, force_triangle=True)
    e2, einf = rel_err(ft, fu)
    assert e2 <= 1e-12 and einf <= 1e-12


def test_rhs_pinned_host_buffers(gpu_lib):
    """Page-locked host arrays take the one-launch path (host reads, product and host writes
    overlapped); the result equals the pageable path bit for bit."""
    import torch
    import fvmgpu as F

    spec = sine_diffusion(64)
    prob = api_problem(spec)
    n = spec.tri.num_points
    u = np.random.default_rng(5).random(n)
    ref = F.fvm_eqs(np.zeros(n), u, prob, 0.0)
    u_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    du_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    u_pin.numpy()[:] = u
    for _ in range(2):
        F.fvm_eqs(du_pin.numpy(), u_pin.numpy(), prob, 0.0)
        assert np.array_equal(du_pin.numpy(), ref)


@pytest.mark.parametrize("make", [lambda: sine_diffusion(64), mixed_annulus, lambda: heat_convection(40)])
def test_rhs_pinned_host_buffers_every_operator_form(gpu_lib, make):
    """The one-launch host-array path on operators with Neumann constants (b), quadratic
    diagonal terms (q), internal Dirichlet and Dudt rows: bit-identical to the pageable path,
    and at t where time factors would enter b."""
    import torch
    import fvmgpu as F

    spec = make()
    prob = api_problem(spec)
    n = spec.tri.num_points
    rng = np.random.default_rng(9)
    u_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    du_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    for _ in range(3):
        u = np.asarray(spec.u0, dtype=np.float64) + rng.standard_normal(n)
        ref = F.fvm_eqs(np.zeros(n), u, prob, 0.25)
        u_pin.numpy()[:] = u
        F.fvm_eqs(du_pin.numpy(), u_pin.numpy(), prob, 0.25)
        assert np.array_equal(du_pin.numpy(), ref)
