"""Pins the oracle's FVMSystem restatement (oracle/fvm_oracle.py: System, system_fvm_eqs,
system_update_dirichlet_nodes) and tests the host classification of system closures
(fvmgpu/forms.py).  CPU only.

Pins, paths relative to the reference project root:
* a system of one component equals the single-equation oracle, which the reference's own
  known-answer tests pin (tests/test_oracle_pins.py);
* the reference's two-component diffusion system (test/test_functions.jl:318-334) solves like
  the single diffusion problem it duplicates (test/equations.jl:106-121);
* the reference's coupled system with an exact solution (test/problem.jl:170-205, the
  Brusselator-type tutorial docs/src/literate_tutorials/reaction_diffusion_brusselator_system_of_pdes.jl):
  the RHS at the exact solution converges to its time derivative at second order.
"""
import numpy as np
import pytest

import fvm_oracle as O
from fvmgpu import forms
from fvmgpu.meshes import triangulate_rectangle
from problems import mixed_annulus, oracle_problem, readme_diffusion, rhs_term_scale


def _tuple_conditions(spec):
    """The spec's conditions with closures of the component tuple u = (u_1,)."""
    wrap = lambda f, p: (lambda x, y, t, u: f(x, y, t, u[0], p))  # noqa: E731
    return O.Conditions(spec.tri, [wrap(f, p) for f, p in zip(spec.bc_fns, spec.bc_params)], list(spec.bc_types),
                        [wrap(f, p) for f, p in zip(spec.ic_fns, spec.ic_params)], spec.dirichlet_nodes,
                        spec.dudt_nodes)


def _one_component_system(spec):
    D, S = spec.D, spec.S

    def q(x, y, t, a, b, g):
        u = a[0] * x + b[0] * y + g[0]
        d = D(x, y, t, u, spec.Dp)
        return (-d * a[0], -d * b[0])

    src = (lambda x, y, t, u: S(x, y, t, u[0], spec.Sp)) if S else None
    return O.System(spec.tri, [_tuple_conditions(spec)], [q], [src], u0=spec.u0[None, :])


def test_system_of_one_component_equals_single_equation_oracle():
    spec = mixed_annulus()
    prob = oracle_problem(spec)
    sys = _one_component_system(spec)
    rng = np.random.default_rng(3)
    for t in (0.0, 0.05):
        u = rng.standard_normal(spec.tri.num_points)
        ref = O.fvm_eqs(prob, u, t)
        got = O.system_fvm_eqs(sys, u[None, :], t)[0]
        scale = rhs_term_scale(prob, u, t)
        assert np.max(np.abs(got - ref) / (np.abs(ref) + scale + 1e-300)) < 1e-13
        # the looped restatement of the single equation agrees as well
        assert np.max(np.abs(O.fvm_eqs_loop(prob, u, t) - got) / (np.abs(ref) + scale + 1e-300)) < 1e-13
    ud = O.system_update_dirichlet_nodes(sys, u[None, :], 0.1)[0]
    assert np.array_equal(ud, O.update_dirichlet_nodes(prob, u, 0.1))


def reference_diffusion_system():
    """example_diffusion_problem_system (test/test_functions.jl:318-334): two copies of the 25 x 25
    diffusion problem with fluxes (-alpha[c]/9, -beta[c]/9)."""
    spec = readme_diffusion(25)
    bc = lambda x, y, t, u: 0.0 * u[0] * u[1]  # noqa: E731
    conds = [O.Conditions(spec.tri, [bc], ["Dirichlet"]) for _ in range(2)]
    q1 = lambda x, y, t, a, b, g: (-a[0] / 9, -b[0] / 9)  # noqa: E731
    q2 = lambda x, y, t, a, b, g: (-a[1] / 9, -b[1] / 9)  # noqa: E731
    sys = O.System(spec.tri, conds, [q1, q2], u0=np.stack([spec.u0, spec.u0]), tf=0.5)
    return sys, spec


def test_reference_diffusion_system_matches_single_problem():
    sys, spec = reference_diffusion_system()
    prob = oracle_problem(spec)
    rng = np.random.default_rng(4)
    u = rng.standard_normal((2, spec.tri.num_points))
    du = O.system_fvm_eqs(sys, u, 0.0)
    for c in range(2):
        ref = O.fvm_eqs(prob, u[c], 0.0)
        assert np.linalg.norm(du[c] - ref) <= 1e-13 * np.linalg.norm(ref)
    # the solutions agree (test/equations.jl:121: every component equals the single problem)
    ts = np.linspace(0.0, 0.05, 6)
    f = lambda v, t: O.system_fvm_eqs(sys, v, t)  # noqa: E731
    cb = lambda v, t: O.system_update_dirichlet_nodes(sys, v, t)  # noqa: E731
    sol, st = O.tsit5_solve(f, sys.u0, 0.0, 0.05, ts, callback=cb)
    ref, _ = O.tsit5_solve(lambda v, t: O.fvm_eqs(prob, v, t), spec.u0, 0.0, 0.05, ts,
                           callback=lambda v, t: O.update_dirichlet_nodes(prob, v, t))
    for c in range(2):
        assert np.max(np.abs(sol[:, c] - ref)) <= 1e-3 * np.max(np.abs(ref))


def brusselator_system(n):
    """The coupled system of test/problem.jl:170-205 with its exact solution
    Phi = exp(-x - y - t/2), Psi = exp(x + y + t/2)."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    phi_bc = [lambda x, y, t, u: -1 / 4 * np.exp(-x - t / 2), lambda x, y, t, u: 1 / 4 * np.exp(-1 - y - t / 2),
              lambda x, y, t, u: np.exp(-1 - x - t / 2), lambda x, y, t, u: -1 / 4 * np.exp(-y - t / 2)]
    psi_bc = [lambda x, y, t, u: np.exp(x + t / 2), lambda x, y, t, u: -1 / 4 * np.exp(1 + y + t / 2),
              lambda x, y, t, u: -1 / 4 * np.exp(1 + x + t / 2), lambda x, y, t, u: np.exp(y + t / 2)]
    conds = [O.Conditions(tri, phi_bc, ["Neumann", "Neumann", "Dirichlet", "Neumann"]),
             O.Conditions(tri, psi_bc, ["Dirichlet", "Neumann", "Neumann", "Dirichlet"])]
    fluxes = [lambda x, y, t, a, b, g: (-a[0] / 4, -b[0] / 4), lambda x, y, t, a, b, g: (-a[1] / 4, -b[1] / 4)]
    sources = [lambda x, y, t, u: u[0] ** 2 * u[1] - 2 * u[0], lambda x, y, t, u: -u[0] ** 2 * u[1] + u[0]]
    P = tri.points
    u0 = np.stack([np.exp(-P[:, 0] - P[:, 1]), np.exp(P[:, 0] + P[:, 1])])
    return O.System(tri, conds, fluxes, sources, u0=u0, tf=5.0)


def test_brusselator_rhs_converges_to_exact_time_derivative():
    errs = []
    for n in (17, 33):
        sys = brusselator_system(n)
        du = O.system_fvm_eqs(sys, sys.u0, 0.0)
        exact = np.stack([-sys.u0[0] / 2, sys.u0[1] / 2])
        on_boundary = np.zeros(sys.tri.num_points, dtype=bool)
        on_boundary[sys.tri.boundary_edges.ravel()] = True
        inner = ~on_boundary
        errs.append(max(np.max(np.abs(du[c, inner] - exact[c, inner]) / np.abs(exact[c, inner])) for c in range(2)))
        # Dirichlet nodes carry du = 0; the update writes the exact boundary values
        ud = O.system_update_dirichlet_nodes(sys, np.zeros_like(sys.u0), 0.0)
        for c in range(2):
            nodes = np.array(sorted(sys.conds[c].dirichlet_nodes))
            assert np.allclose(ud[c, nodes], sys.u0[c, nodes], rtol=1e-14)
            assert np.all(du[c, nodes] == 0.0)
    assert errs[0] < 1e-2
    assert errs[0] / errs[1] > 3.5  # second order on the interior nodes


# ---- host classification of system closures ------------------------------------------------
def test_monomial_basis():
    for N, M in ((1, 4), (2, 10), (3, 20), (4, 35), (8, 165)):
        e = forms.monomials(N)
        assert e.shape == (M, N) and np.all(e.sum(axis=1) <= 3)
        assert len({tuple(r) for r in e}) == M and not np.any(e[0])


def test_classify_system_sources():
    x = np.linspace(-1, 1, 40)
    y = np.linspace(0, 2, 40)
    b, d = 0.04, 0.1
    e, c = forms.classify_system_poly(lambda x, y, t, u: b * (1 - u[0]) - u[0] * u[1] ** 2, x, y, 0.0, 2, "u_S")
    got = {tuple(k): c[:, m] for m, k in enumerate(e)}
    assert set(got) == {(0, 0), (1, 0), (1, 2)}
    assert np.allclose(got[(0, 0)], b, rtol=1e-13) and np.allclose(got[(1, 0)], -b, rtol=1e-13)
    assert np.allclose(got[(1, 2)], -1, rtol=1e-13)
    e, c = forms.classify_system_poly(lambda x, y, t, u: -d * u[1] + u[0] * u[1] ** 2, x, y, 0.0, 2, "v_S")
    assert {tuple(k) for k in e} == {(0, 1), (1, 2)}
    e, c = forms.classify_system_poly(lambda x, y, t, u: x * u[0] ** 2 * u[1] - 2 * u[0] + y, x, y, 0.0, 2, "S")
    got = {tuple(k): c[:, m] for m, k in enumerate(e)}
    assert np.allclose(got[(2, 1)], x, atol=1e-13) and np.allclose(got[(0, 0)], y, atol=1e-13)
    e, c = forms.classify_system_poly(lambda x, y, t, u: 0.0 * x, x, y, 0.0, 3, "zero")
    assert e.shape == (0, 3) and c.shape == (40, 0)
    # a closure that destructures the tuple, called per point when it does not take arrays
    e, c = forms.classify_system_poly(lambda x, y, t, uv: (uv[0] if x < 0 else 2.0) * uv[1], x, y, 0.0, 2, "branch")
    got = {tuple(k): c[:, m] for m, k in enumerate(e)}
    assert np.allclose(got[(1, 1)], np.where(x < 0, 1.0, 0.0), atol=1e-12)
    assert np.allclose(got[(0, 1)], np.where(x < 0, 0.0, 2.0), atol=1e-12)
    for bad in (lambda x, y, t, u: np.exp(u[0]), lambda x, y, t, u: u[0] ** 4, lambda x, y, t, u: t * u[1],
                lambda x, y, t, u: u[0] * u[1] * u[1] * u[0], lambda x, y, t, u: 1 / (x - x) + u[0]):
        with pytest.raises(forms.UnsupportedFormError):
            forms.classify_system_poly(bad, x, y, 0.0, 2, "bad")
    with pytest.raises(forms.UnsupportedFormError):  # Neumann values must be affine
        forms.classify_system_poly(lambda x, y, t, u: u[0] * u[1], x, y, 0.0, 2, "Neumann", max_degree=1)
    with pytest.raises(forms.UnsupportedFormError):  # Dirichlet values are functions of (x, y)
        forms.classify_system_poly(lambda x, y, t, u: x + u[0], x, y, 0.0, 2, "Dirichlet", max_degree=0)


def test_classify_system_fluxes():
    x = np.linspace(-1, 1, 30)
    y = np.linspace(0, 1, 30)
    D = forms.classify_system_flux(lambda x, y, t, a, b, g: (-a[1] * (1 + x), -b[1] * (1 + x)), x, y, 0.0, 2)
    assert np.allclose(D[1], 1 + x, rtol=1e-15) and not np.any(D[0])
    q = lambda x, y, t, a, b, g: (-(2 * a[0] - 0.5 * y * a[2]), -(2 * b[0] - 0.5 * y * b[2]))  # noqa: E731
    D = forms.classify_system_flux(q, x, y, 0.0, 3)
    assert np.allclose(D[0], 2.0) and np.allclose(D[2], -0.5 * y) and not np.any(D[1])
    for bad in (lambda x, y, t, a, b, g: (-a[0] * (a[0] * x + g[0]), -b[0]),  # D(u): nonlinear
                lambda x, y, t, a, b, g: (-a[0], -2 * b[0]),                  # anisotropic
                lambda x, y, t, a, b, g: (-a[0] + 0.1, -b[0]),                # advection-like constant
                lambda x, y, t, a, b, g: (-a[0] * (1 + t), -b[0] * (1 + t)),  # time dependent
                lambda x, y, t, a, b, g: -a[0]):                              # not a pair
        with pytest.raises(forms.UnsupportedFormError):
            forms.classify_system_flux(bad, x, y, 0.0, 2)


# ---- Jacobian prototype (src/solve.jl:50-131; test/test_functions.jl:749-793) ---------------
def _reference_test_matrix(tri, N):
    """The dense matrix the reference's test_jacobian_sparsity builds (test/test_functions.jl:
    749-793): for each solid vertex i and each j in (i, neighbours...), all (x, y) with x among
    i's unknowns and y among j's."""
    n = tri.num_points
    A = np.zeros((n * N, n * N))
    nb = [set() for _ in range(n)]
    for a, b, c in tri.triangles:
        for u, v in ((a, b), (b, c), (c, a)):
            nb[u].add(v)
            nb[v].add(u)
    for i in np.nonzero(tri.has_vertex())[0]:
        for j in [i, *nb[i]]:
            A[i * N:(i + 1) * N, j * N:(j + 1) * N] = 1.0
    return A


@pytest.mark.parametrize("N", [None, 1, 2, 3])
def test_jacobian_sparsity_matches_reference(N):
    import fvmgpu as F
    from fvmgpu.meshes import triangulate_annulus

    for tri in (triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 7, 9, single_boundary=False),
                triangulate_annulus(0.5, 1.0, 4, 16, nsegments=4)):
        J = F.jacobian_sparsity(tri, N)
        K = 1 if N is None else N
        assert J.shape == (tri.num_points * K,) * 2 and J.format == "csc"
        assert np.all(J.data == 1.0)
        got = set(zip(*J.nonzero()))
        entries, dim = O.jacobian_sparsity(tri, N)
        assert dim == J.shape[0] and got == entries
        assert np.array_equal(J.toarray(), _reference_test_matrix(tri, K))


# ---- output side: compute_flux, pl_interpolate, two_point_interpolant ------------------------
class _Mesh:
    """Host stand-in for FVMGeometry: the triangulation and the geometry rows the library
    exports (s1..s9, dual-edge midpoints, normals, lengths), here from the oracle's geometry."""

    def __init__(self, tri):
        g = O.Geometry(tri.points, tri.triangles)
        self.triangulation = tri
        self.props_array = np.hstack([g.s, g.mid.reshape(-1, 6), g.nrm.reshape(-1, 6), g.length])


def _edges(tri):
    e = set()
    for a, b, c in tri.triangles:
        e |= {(int(a), int(b)), (int(b), int(c)), (int(c), int(a))}
    return sorted(e)


def test_compute_flux_and_interpolation_match_oracle():
    """test/test_functions.jl:660-747: every solid edge's flux q . n at its midpoint, the normal
    pointing to the edge's right, from the triangle on that side (the other one on the
    boundary); pl_interpolate reproduces the linear interpolant."""
    import fvmgpu as F

    spec = mixed_annulus()
    mesh = _Mesh(spec.tri)
    types = tuple(getattr(F, t) for t in spec.bc_types)
    BCs = F.BoundaryConditions(mesh, tuple(spec.bc_fns), types, parameters=tuple(spec.bc_params))
    prob = F.FVMProblem(mesh, BCs, diffusion_function=spec.D, diffusion_parameters=spec.Dp, initial_condition=spec.u0,
                        final_time=1.0)
    oprob = oracle_problem(spec)
    u = np.random.default_rng(6).standard_normal(spec.tri.num_points)
    for (i, j) in _edges(spec.tri)[::3]:
        got = F.compute_flux(prob, i, j, u, 2.5)
        assert got == O.compute_flux(oprob, i, j, u, 2.5)
        # the reference test's own construction for interior edges: the triangle (j, i, k)
        k = O.adjacent(spec.tri, j, i)
        if k is not None:
            p, q = spec.tri.points[i], spec.tri.points[j]
            a, b, c = O._abg_at(oprob, (j, i, k), u)
            mx, my = (p + q) / 2
            qv = oprob.flux(mx, my, 2.5, a, b, c)
            n = np.array([q[1] - p[1], -(q[0] - p[0])]) / np.linalg.norm(q - p)
            assert np.isclose(got, qv[0] * n[0] + qv[1] * n[1], rtol=1e-12, atol=1e-14)
    for T in spec.tri.triangles[::7]:
        x, y = spec.tri.points[T].mean(axis=0)
        for rot in ((0, 1, 2), (1, 2, 0), (2, 0, 1)):
            Tr = tuple(int(T[r]) for r in rot)
            assert F.pl_interpolate(prob, Tr, u, x, y) == O.pl_interpolate(oprob, Tr, u, x, y)
        # the interpolant reproduces the vertex values (test/geometry.jl:23-75 identities)
        for v in T:
            assert np.isclose(F.pl_interpolate(prob, tuple(T), u, *spec.tri.points[v]), u[v], atol=1e-12)
    i, j = (int(v) for v in spec.tri.triangles[0][:2])
    pi, pj = spec.tri.points[i], spec.tri.points[j]
    m = 0.25 * pi + 0.75 * pj
    assert np.isclose(F.two_point_interpolant(mesh, u, i, j, *m), 0.25 * u[i] + 0.75 * u[j], rtol=1e-13)
    with pytest.raises(ValueError):
        F.pl_interpolate(prob, (0, 0, 0), u, 0.0, 0.0)


def test_compute_flux_of_a_system():
    """compute_flux on a system returns one value per component; a component's value equals the
    single problem's (test/test_functions.jl:703-704)."""
    import fvmgpu as F

    sys, spec = reference_diffusion_system()

    class _Sys:  # host stand-in: compute_flux reads mesh and flux_functions only
        mesh = _Mesh(spec.tri)
        flux_functions = [lambda x, y, t, a, b, g: (-a[0] / 9, -b[0] / 9),
                          lambda x, y, t, a, b, g: (-a[1] / 9, -b[1] / 9)]

    u = np.random.default_rng(7).standard_normal((2, spec.tri.num_points))
    oprob = oracle_problem(spec)
    for (i, j) in _edges(spec.tri)[::11]:
        got = F.compute_flux(_Sys, i, j, u, 0.0)
        assert got == O.compute_flux(sys, i, j, u, 0.0)
        for c in range(2):
            assert np.isclose(got[c], O.compute_flux(oprob, i, j, u[c], 0.0), rtol=1e-13, atol=1e-15)
    T = tuple(int(v) for v in spec.tri.triangles[5])
    x, y = spec.tri.points[list(T)].mean(axis=0)
    assert np.array_equal(F.pl_interpolate(_Sys, T, u, x, y), O.pl_interpolate(sys, T, u, x, y))


def test_system_fit_keeps_position_independent_coefficients_exact():
    """Coefficients that do not depend on (x, y) come out as one value at every point, whether or
    not another coefficient depends on (x, y); the constant term is the closure's own value."""
    x = np.linspace(-1, 1, 2000)
    y = np.linspace(0, 1, 2000)
    e, c = forms.classify_system_poly(lambda x, y, t, u: 0.04 * (1 - u[0]) - u[0] * u[1] ** 2, x, y, 0.0, 2, "S")
    assert all(np.unique(c[:, k]).size == 1 for k in range(c.shape[1]))
    f = lambda x, y, t, u: (1 + x * x) * u[0] * u[1] - 0.3 * u[1] ** 3 + 0.04 * u[0] - y  # noqa: E731
    e, c = forms.classify_system_poly(f, x, y, 0.0, 2, "S")
    got = {tuple(k): c[:, m] for m, k in enumerate(e)}
    assert np.unique(got[(1, 0)]).size == 1 and np.unique(got[(0, 3)]).size == 1
    assert np.allclose(got[(1, 0)], 0.04, rtol=1e-13) and np.allclose(got[(0, 3)], -0.3, rtol=1e-13)
    assert np.array_equal(got[(0, 0)], -y)  # the value at u = 0, exactly
    assert np.allclose(got[(1, 1)], 1 + x * x, rtol=1e-12)


def test_decoupled_system_equals_its_single_problems():
    """Two components on one annulus, each with its own conditions (component 0: the mixed
    Dirichlet / Dudt / Neumann / Constrained layout with internal nodes; component 1: a different
    layout), diffusion and source, not coupled: each row of the system RHS and of the Dirichlet
    update equals its own single problem's (merge_problem_conditions keeps conditions per
    component, src/problem.jl:336-365)."""
    from problems import Spec

    a = mixed_annulus()
    types_b = ("Neumann", "Dirichlet", "Dudt", "Neumann", "Constrained", "Neumann", "Dirichlet", "Neumann")
    b = Spec(a.tri, a.bc_fns[::-1], types_b, a.bc_params[::-1],
             D=lambda x, y, t, u, p: 2.0 + y * y + 0.0 * u, S=lambda x, y, t, u, p: -u + 0.5 * u * u, u0=a.u0[::-1].copy())
    specs = (a, b)
    probs = [oracle_problem(s) for s in specs]

    def comp(s, c):
        wrap = lambda f, p: (lambda x, y, t, u: f(x, y, t, u[c], p))  # noqa: E731
        cond = O.Conditions(s.tri, [wrap(f, p) for f, p in zip(s.bc_fns, s.bc_params)], list(s.bc_types),
                            [wrap(f, p) for f, p in zip(s.ic_fns, s.ic_params)], s.dirichlet_nodes, s.dudt_nodes)

        def q(x, y, t, al, be, ga):
            d = s.D(x, y, t, al[c] * x + be[c] * y + ga[c], s.Dp)
            return (-d * al[c], -d * be[c])

        src = lambda x, y, t, u: s.S(x, y, t, u[c], s.Sp)  # noqa: E731
        return cond, q, src

    parts = [comp(s, c) for c, s in enumerate(specs)]
    sys = O.System(a.tri, [p[0] for p in parts], [p[1] for p in parts], [p[2] for p in parts])
    rng = np.random.default_rng(12)
    u = rng.standard_normal((2, a.tri.num_points))
    du = O.system_fvm_eqs(sys, u, 0.0)
    ud = O.system_update_dirichlet_nodes(sys, u, 0.0)
    for c in range(2):
        ref = O.fvm_eqs(probs[c], u[c], 0.0)
        scale = rhs_term_scale(probs[c], u[c], 0.0)
        assert np.max(np.abs(du[c] - ref) / (np.abs(ref) + scale + 1e-300)) < 1e-13
        assert np.array_equal(ud[c], O.update_dirichlet_nodes(probs[c], u[c], 0.0))
        assert np.array_equal(sys.code[c], probs[c].code)


@pytest.mark.parametrize("seed", range(6))
def test_classify_recovers_random_polynomials(seed):
    """Seeded random polynomials of total degree <= 3 in N <= 4 components, some coefficients
    depending on (x, y), others constant: the classifier returns exactly their monomials, the
    coefficients to 1e-12, and the constant ones as one value at every point."""
    rng = np.random.default_rng(100 + seed)
    N = int(rng.integers(1, 5))
    basis = forms.monomials(N)
    pick = rng.choice(basis.shape[0], size=int(rng.integers(1, min(6, basis.shape[0]) + 1)), replace=False)
    terms = []
    for k in pick:
        if rng.random() < 0.5:
            c0 = float(rng.normal())
            terms.append((tuple(basis[k]), lambda x, y, c0=c0: c0 + 0.0 * x, True))
        else:
            a, b = rng.normal(size=2)
            terms.append((tuple(basis[k]), lambda x, y, a=a, b=b: a * x + b * y * y + 1.0, False))

    def f(x, y, t, u):
        out = 0.0 * x
        for e, c, _ in terms:
            m = c(x, y)
            for q, k in enumerate(e):
                m = m * u[q] ** k
            out = out + m
        return out

    x = rng.uniform(-1, 1, 300)
    y = rng.uniform(-1, 1, 300)
    e, c = forms.classify_system_poly(f, x, y, 0.0, N, "random")
    got = {tuple(k): c[:, m] for m, k in enumerate(e)}
    assert set(got) == {t[0] for t in terms}
    for ek, cf, const in terms:
        ref = cf(x, y)
        assert np.max(np.abs(got[ek] - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref))), ek
        if const:
            assert np.unique(got[ek]).size == 1, ek


def test_system_fit_rejects_small_t_dependence_and_keeps_small_varying_coefficients():
    """The fit's acceptance is relative to the size of the evaluated terms: a t-dependence of
    1e-9 of the value is rejected.  Snapping to one value is relative to each coefficient's own
    size: a coefficient that varies with (x, y) stays varying however small it is next to the
    others."""
    x = np.linspace(-1, 1, 500)
    y = np.linspace(0, 1, 500)
    with pytest.raises(forms.UnsupportedFormError):
        forms.classify_system_poly(lambda x, y, t, u: u[0] * (1 + 1e-9 * t) + 0.0 * x, x, y, 0.0, 2, "S")
    e, c = forms.classify_system_poly(lambda x, y, t, u: 5.0 * u[0] ** 2 + 1e-9 * (1 + x) * u[1], x, y, 0.0, 2, "S")
    got = {tuple(k): c[:, m] for m, k in enumerate(e)}
    assert np.unique(got[(0, 1)]).size > 1  # not flattened
    assert np.allclose(got[(0, 1)], 1e-9 * (1 + x), rtol=1e-6, atol=1e-14)  # fit noise ~1e-16 of 5
    assert np.unique(got[(2, 0)]).size == 1
