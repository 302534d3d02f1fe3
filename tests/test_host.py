"""Host-side logic without a GPU: mesh generators, condition merging, closure classification."""
import numpy as np
import pytest

import fvm_oracle as O
from fvmgpu import forms
from fvmgpu.api import BoundaryConditions, Conditions, InternalConditions, _saveat_times
from fvmgpu.meshes import triangulate_annulus, triangulate_disk, triangulate_rectangle
import fvmgpu.api as api


class _Mesh:
    def __init__(self, tri):
        self.triangulation = tri


def test_rectangle_numbering_matches_reference_tests():
    tri = triangulate_rectangle(0.0, 2.0, 0.0, 5.0, 12, 19, single_boundary=False)
    P = tri.points
    # vertex i + (j-1) nx (1-based) = (i-1) + (j-1) nx (0-based), x fastest (test_functions.jl:112)
    assert np.allclose(P[6 + 3 * 12], [6 * 2.0 / 11, 3 * 5.0 / 18])
    t200 = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 200, 200)
    assert (0, 1, 200) in set(map(tuple, t200.triangles.tolist()))  # test/equations.jl:42
    assert tri.num_triangles == 2 * 11 * 18 and tri.num_boundary_edges == 2 * 11 + 2 * 18
    assert [len(s) for s in tri.boundary_nodes] == [12, 19, 12, 19]
    assert np.all(P[tri.boundary_nodes[0], 1] == 0.0) and np.all(P[tri.boundary_nodes[1], 0] == 2.0)
    assert np.all(P[tri.boundary_nodes[2], 1] == 5.0) and np.all(P[tri.boundary_nodes[3], 0] == 0.0)
    single = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 5, 5, single_boundary=True)
    assert single.num_ghost_vertices == 1 and single.boundary_nodes[0][0] == single.boundary_nodes[0][-1]


def test_triangles_ccw_and_boundary_adjacency():
    for tri in (triangulate_rectangle(0, 1, 0, 1, 7, 9), triangulate_annulus(0.5, 1.0, 5, 24),
                triangulate_disk(400, 32, seed=1)):
        P, T = tri.points, tri.triangles
        det = ((P[T[:, 1], 0] - P[T[:, 0], 0]) * (P[T[:, 2], 1] - P[T[:, 0], 1])
               - (P[T[:, 1], 1] - P[T[:, 0], 1]) * (P[T[:, 2], 0] - P[T[:, 0], 0]))
        assert np.all(det > 0)
        tset = {tuple(t) for t in T.tolist()}
        for (i, j), k in zip(tri.boundary_edges, tri.boundary_adjacent):
            assert (i, j, k) in tset or (j, k, i) in tset or (k, i, j) in tset
    d = triangulate_disk(1000, 64, seed=0)
    assert d.num_triangles == 2 * d.num_points - 64 - 2
    assert d.num_boundary_edges == 64


def test_conditions_merge_matches_oracle_bit_exact():
    tri = triangulate_annulus(0.5, 1.0, 6, 32, nsegments=4)
    types = ("Dirichlet", "Dudt", "Neumann", "Constrained", "Neumann", "Dirichlet", "Dudt", "Neumann")
    fns = tuple((lambda x, y, t, u, p, k=k: k + 0.0 * x) for k in range(8))
    mesh = _Mesh(tri)
    bc = BoundaryConditions(mesh, fns, tuple(getattr(api, t) for t in types))
    ic = InternalConditions((lambda x, y, t, u, p: x,), dirichlet_nodes={40: 0, 0: 0}, dudt_nodes={41: 0})
    c = Conditions(mesh, bc, ic)
    oc = O.Conditions(tri, [lambda x, y, t, u: x] * 8, list(types), [lambda x, y, t, u: x], {40: 0, 0: 0}, {41: 0})
    assert c.neumann_edges == oc.neumann_edges
    assert c.constrained_edges == oc.constrained_edges
    assert c.dirichlet_nodes == oc.dirichlet_nodes
    assert c.dudt_nodes == oc.dudt_nodes
    hv = tri.has_vertex()
    code, fidx = c.vertex_tables(hv)
    ocode, ofidx = oc.vertex_tables(tri.num_points, hv)
    assert np.array_equal(code, ocode) and np.array_equal(fidx, ofidx)
    assert np.array_equal(c.neumann_table(tri.boundary_edges), oc.edge_tables(tri.boundary_edges))


def test_boundary_conditions_argument_checks():
    tri = triangulate_rectangle(0, 1, 0, 1, 4, 4, single_boundary=False)
    mesh = _Mesh(tri)
    f = lambda x, y, t, u, p: x  # noqa: E731
    with pytest.raises(AssertionError):
        BoundaryConditions(mesh, f, api.Dirichlet)  # 4 boundary parts need 4 conditions
    with pytest.raises(AssertionError):
        BoundaryConditions(mesh, (f,) * 4, (api.Dirichlet,) * 3)
    bc = BoundaryConditions(triangulate_rectangle(0, 1, 0, 1, 4, 4, single_boundary=True) and
                            _Mesh(triangulate_rectangle(0, 1, 0, 1, 4, 4, single_boundary=True)), f, api.Dirichlet,
                            parameters=(0.3, 0.6, -1.0))
    assert bc.functions[0].parameters == (0.3, 0.6, -1.0)  # a lone function keeps its tuple p


def test_form_classification():
    x = np.linspace(0, 1, 50)
    y = np.linspace(1, 2, 50)
    c, d = forms.classify_xytu(lambda x, y, t, u: 1 / 9 + 0.0 * x, x, y, 0.0, "D")
    assert d == 0 and np.allclose(c[:, 0], 1 / 9)
    c, d = forms.classify_xytu(lambda x, y, t, u: x * y + 2.0 * u, x, y, 0.0, "a")
    assert d == 1 and np.allclose(c[:, 0], x * y) and np.allclose(c[:, 1], 2.0)
    c, d = forms.classify_xytu(lambda x, y, t, u: u * (1 - u), x, y, 0.0, "S")
    assert d == 2 and np.allclose(c, [[0.0, 1.0, -1.0]] * 50)
    c, d = forms.classify_xytu(lambda x, y, t, u: 50.0 if y <= 1.5 else 0.0, x, y, 0.0, "branching closure")
    assert d == 0 and np.allclose(c[:, 0], np.where(y <= 1.5, 50.0, 0.0))
    for bad in (lambda x, y, t, u: np.exp(u), lambda x, y, t, u: t + 0.0 * x, lambda x, y, t, u: u ** 3,
                lambda x, y, t, u: 1 / (x - x)):
        with pytest.raises(forms.UnsupportedFormError):
            forms.classify_xytu(bad, x, y, 0.0, "bad")
    D = forms.classify_flux(lambda x, y, t, a, b, g: (-(1 + x) * a, -(1 + x) * b), x, y, 0.0)
    assert np.allclose(D, 1 + x)
    with pytest.raises(forms.UnsupportedFormError):
        forms.classify_flux(lambda x, y, t, a, b, g: (-a * (a * x + b * y + g), -b), x, y, 0.0)


def test_saveat_times_follow_julia_ranges():
    ts = _saveat_times(0.001, 0.0, 0.5)
    assert ts.size == 501 and ts[0] == 0.0 and abs(ts[-1] - 0.5) < 1e-12
    assert np.array_equal(_saveat_times([0.1, 0.2], 0.0, 1.0), [0.1, 0.2])
    assert np.array_equal(_saveat_times(None, 0.0, 1.0), [0.0, 1.0])


def test_problems_and_system_conditions_without_a_device():
    """An FVMProblem is built without touching the device (its closures are classified on first
    use); the conditions of a system merge as merge_problem_conditions does
    (test/problem.jl:170-260: cnum_fncs == (0, 4), map_fidx, the merged function list, each
    component's Neumann / Dirichlet tables)."""
    import numpy as np

    from fvmgpu import api
    from fvmgpu.meshes import triangulate_rectangle

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 10, 10, single_boundary=False)

    class Mesh:  # a host stand-in: BoundaryConditions and FVMProblem read the triangulation only
        triangulation = tri

    phi = (lambda x, y, t, u, p: -0.25 * np.exp(-x - t / 2), lambda x, y, t, u, p: 0.25 * np.exp(-1 - y - t / 2),
           lambda x, y, t, u, p: np.exp(-1 - x - t / 2), lambda x, y, t, u, p: -0.25 * np.exp(-y - t / 2))
    psi = (lambda x, y, t, u, p: np.exp(x + t / 2), lambda x, y, t, u, p: -0.25 * np.exp(1 + y + t / 2),
           lambda x, y, t, u, p: -0.25 * np.exp(1 + x + t / 2), lambda x, y, t, u, p: np.exp(y + t / 2))
    N_, D_ = api.Neumann, api.Dirichlet
    pbc = api.BoundaryConditions(Mesh, phi, (N_, N_, D_, N_))
    sbc = api.BoundaryConditions(Mesh, psi, (D_, N_, N_, D_))
    q1 = lambda x, y, t, a, b, g, p: (-a[0] / 4, -b[0] / 4)  # noqa: E731
    q2 = lambda x, y, t, a, b, g, p: (-a[1] / 4, -b[1] / 4)  # noqa: E731
    S1 = lambda x, y, t, u, p: u[0] ** 2 * u[1] - 2 * u[0]  # noqa: E731
    S2 = lambda x, y, t, u, p: -u[0] ** 2 * u[1] + u[0]  # noqa: E731
    u0 = np.zeros(tri.num_points)
    p1 = api.FVMProblem(Mesh, pbc, flux_function=q1, source_function=S1, initial_condition=u0, final_time=5.0)
    p2 = api.FVMProblem(Mesh, sbc, flux_function=q2, source_function=S2, initial_condition=u0, final_time=5.0)
    assert p1._h is None and not p1._built  # nothing classified, nothing on the device
    conds, cnum, fns, srcs, fluxes = api.merge_problem_conditions((p1, p2))
    assert cnum == (0, 4) and len(fns) == 8
    assert conds[0] is p1.conditions and conds[1] is p2.conditions
    for k in range(4):
        assert fns[k] is p1.conditions.functions[k] and fns[4 + k] is p2.conditions.functions[k]
    x, y, t = 0.3, 0.7, 0.9
    for (i, j), f in p2.conditions.neumann_edges.items():
        assert fns[f + cnum[1]](x, y, t, (1.0, 2.0)) == p2.conditions.functions[f](x, y, t, (1.0, 2.0))
    assert srcs[0](x, y, t, (2.0, 3.0)) == S1(x, y, t, (2.0, 3.0), None)
    assert fluxes[1](x, y, t, (1.0, 2.0), (3.0, 4.0), (5.0, 6.0)) == (-0.5, -1.0)
    # component tables: Phi is Neumann on three sides and Dirichlet on the top, Psi the reverse pattern
    assert len(conds[0].dirichlet_nodes) == 10 and len(conds[1].dirichlet_nodes) == 19
    assert len(conds[0].neumann_edges) == 27 and len(conds[1].neumann_edges) == 18


def test_construct_flux_function():
    """test/problem.jl:152-160: a given flux is returned as it is; otherwise the diffusion flux
    -D(x, y, t, alpha x + beta y + gamma, Dp) (alpha, beta)."""
    import numpy as np

    import fvmgpu as F

    q = lambda x, y, t, a, b, g, p: (a, b)  # noqa: E731
    assert F.construct_flux_function(q, None, None) is q
    D = lambda x, y, t, u, p: x + y + t + u + p[1]  # noqa: E731
    Dp = (0.2, 5.73)
    _q = F.construct_flux_function(None, D, Dp)
    x, y, t, a, b, g = np.random.default_rng(3).random(6)
    u = a * x + b * y + g
    assert _q(x, y, t, a, b, g, None) == (-a * D(x, y, t, u, Dp), -b * D(x, y, t, u, Dp))


def test_classify_linear_flux_advection_and_rejections():
    """The advection-diffusion flux of the reference's tutorial, q = nu u - D grad u with
    u = alpha x + beta y + gamma, is linear in (alpha, beta, gamma): M = (nu_x x - D, nu_x y, nu_x,
    nu_y x, nu_y y - D, nu_y).  Non-linear or t-dependent fluxes are rejected."""
    from fvmgpu import forms

    x = np.linspace(-1, 1, 50)
    y = np.linspace(0, 2, 50)
    D, nu = 0.02, 0.05

    def q(x, y, t, a, b, g, p=None):
        u = a * x + b * y + g
        return nu * u - D * a, -D * b

    M = forms.classify_linear_flux(q, x, y, 0.0)
    ref = np.stack([nu * x - D, nu * y, nu + 0 * x, 0 * x, 0 * x - D, 0 * x], axis=1)
    assert np.allclose(M, ref, rtol=1e-13, atol=1e-15)
    for bad in (lambda x, y, t, a, b, g: (a * a, b), lambda x, y, t, a, b, g: (a * (1 + t), b),
                lambda x, y, t, a, b, g: (a + 1.0, b)):
        with pytest.raises(forms.UnsupportedFormError):
            forms.classify_linear_flux(bad, x, y, 0.0)


def test_time_factor_fit_recovers_the_device_set():
    """Constant terms A(x, y) + tau(t) B(x, y) with tau = exp(a (t - t0)) or a quadratic in
    t - t0 are fitted to within rounding (the annulus tutorial's 50 (1 - exp(-t/2)), the
    Brusselator's exp(-x - t/2)); other t dependence, or t in the u-dependent terms, is rejected."""
    from fvmgpu import forms

    x = np.linspace(0, 1, 40)
    y = np.cos(3 * x)
    cases = [(lambda x, y, t, u: 50 * (1 - np.exp(-t / 2)) + 0 * x, 0.0, 2.0, 1.0, -0.5),
             (lambda x, y, t, u: -0.25 * np.exp(-x - t / 2), 0.0, 1.0, 1.0, -0.5),
             (lambda x, y, t, u: (2 - t) * x + 0.3 * u, 0.5, 1.5, 2.0, None),
             (lambda x, y, t, u: (1 + 0.3 * t + 0.2 * t * t) * np.sin(3 * x) - u * u, 0.5, 1.5, 2.0, None),
             (lambda x, y, t, u: np.exp(0.7 * t) * y, 0.0, 5.0, 1.0, 0.7)]
    for f, t0, tf, kind, a in cases:
        c, deg, tp = forms.classify_xytu(f, x, y, t0, "f", tf=tf, time=True)
        tau, B = tp
        assert tau[0] == kind and tau[1] == t0
        if a is not None:
            assert abs(tau[2] - a) <= 1e-12 * abs(a)
        for t in np.linspace(t0, tf + 1, 7):
            want = f(x, y, t, 0.0)
            assert np.max(np.abs(c[:, 0] + tau(t) * B - want)) <= 1e-13 * max(1.0, np.max(np.abs(want)))
    c, deg, tp = forms.classify_xytu(lambda x, y, t, u: x + 2 * u, x, y, 0.0, "f", tf=1.0, time=True)
    assert tp is None and deg == 1
    for bad in (lambda x, y, t, u: np.sin(t) * x, lambda x, y, t, u: t * u, lambda x, y, t, u: np.exp(-t) * x + t * y):
        with pytest.raises(forms.UnsupportedFormError):
            forms.classify_xytu(bad, x, y, 0.0, "g", tf=1.0, time=True)
    with pytest.raises(forms.UnsupportedFormError, match="depends on t"):
        forms.classify_xytu(lambda x, y, t, u: np.exp(-t) * x, x, y, 0.0, "g")  # time not allowed here


def test_time_factors_merge_across_closures():
    """Closures with the same factor share one descriptor row (the Brusselator's three
    exp(-t/2) sides), each kind of value in its own array; more than eight factors are refused."""
    from fvmgpu import forms
    from fvmgpu.api import _TimeParts

    parts = _TimeParts({"time_dirichlet": 5, "time_neumann": 4, "time_source": 5, "time_dudt": 5})
    x = np.linspace(0, 1, 2)
    for k, f in enumerate((lambda x, y, t, u: np.exp(-x - t / 2), lambda x, y, t, u: -np.exp(-1 - x - t / 2))):
        _, _, (tau, B) = forms.classify_xytu(f, x, x, 0.0, "f", tf=1.0, time=True)
        sel = np.zeros(4, dtype=bool)
        sel[2 * k:2 * k + 2] = True
        parts.add("time_neumann", tau, sel, B)
    assert len(parts.factors) == 1 and np.all(parts.values["time_neumann"][0] != 0)
    for g in range(7):
        parts.add("time_source", forms.TimeFactor(2, 0.0, g + 1.0), np.ones(5, dtype=bool), np.ones(5))
    with pytest.raises(forms.UnsupportedFormError, match="time factors"):
        parts.add("time_source", forms.TimeFactor(2, 0.0, 99.0), np.ones(5, dtype=bool), np.ones(5))


def test_system_time_factor_fit():
    """System closures (the Brusselator's boundary values): the constant term's factor is fitted
    and the remaining polynomial is the static part; t in a component-dependent term is refused."""
    from fvmgpu import forms

    x = np.linspace(0, 1, 12)
    y = x[::-1].copy()
    f = lambda x, y, t, u: -0.25 * np.exp(1 + y + t / 2) + 0.3 * u[0]  # noqa: E731
    e, c, (tau, B) = forms.classify_system_poly(f, x, y, 0.0, 2, "f", max_degree=1, tf=5.0, time=True)
    assert e.tolist() == [[1, 0]] and np.allclose(c[:, 0], 0.3, rtol=1e-13)
    assert tau[0] == 1.0 and abs(tau[2] - 0.5) <= 1e-12
    for t in (0.0, 1.3, 5.0):
        assert np.allclose(tau(t) * B, -0.25 * np.exp(1 + y + t / 2), rtol=1e-13, atol=0)
    e, c, tp = forms.classify_system_poly(lambda x, y, t, u: u[0] ** 2 * u[1] - 2 * u[0], x, y, 0.0, 2, "S",
                                          tf=5.0, time=True)
    assert tp is None and e.tolist() == [[1, 0], [2, 1]]
    with pytest.raises(forms.UnsupportedFormError):
        forms.classify_system_poly(lambda x, y, t, u: np.exp(-t) * u[0] + x, x, y, 0.0, 2, "g", tf=1.0, time=True)


def test_classification_checks_every_point():
    """Only two of the verification probes run at every point; they still catch a t dependence
    or a non-polynomial u dependence confined to one point off the subsample, and a time factor
    there is fitted at every point."""
    from fvmgpu import forms

    n = 40_000
    x = np.linspace(0.0, 1.0, n)
    y = np.zeros(n)
    x5 = x[5]  # the subsample takes every 9th point: 0, 9, 18, ...
    odd = lambda x: np.where(x == x5, 1.0, 0.0)  # noqa: E731
    with pytest.raises(forms.UnsupportedFormError, match="depends on t"):
        forms.classify_xytu(lambda x, y, t, u: x + odd(x) * t, x, y, 0.0, "f")
    with pytest.raises(forms.UnsupportedFormError, match="polynomial"):
        forms.classify_xytu(lambda x, y, t, u: x + odd(x) * np.exp(u), x, y, 0.0, "f")
    c, deg, (tau, B) = forms.classify_xytu(lambda x, y, t, u: x + odd(x) * np.exp(-t), x, y, 0.0, "f", tf=1.0,
                                           time=True)
    assert deg == 0 and tau[0] == 1.0 and abs(tau[2] + 1.0) < 1e-12
    assert abs(B[5] - 1.0) < 1e-12 and np.all(B[np.arange(n) != 5] == 0)


def test_time_factor_fit_with_an_infinite_final_time():
    """A steady problem's final time is Inf: the time-factor fit then samples t0 + [0, 1] and
    still recovers a factor, or finds none for values that do not depend on t."""
    x = np.linspace(0.0, 1.0, 7)
    fit = forms.fit_time_factor(lambda t: 2.0 + x * np.exp(-0.5 * t), 0.0, np.inf, "test")
    assert fit is not None
    A, tau, B = fit
    for t in (0.0, 0.3, 4.0):
        assert np.allclose(A + tau(t) * B, 2.0 + x * np.exp(-0.5 * t), rtol=1e-12, atol=1e-12)
    assert forms.fit_time_factor(lambda t: 1.0 + x, 0.0, np.inf, "test") is None


def test_steady_types_without_a_device():
    """SteadyFVMProblem wraps problems and systems only; the steady methods' defaults are
    SteadyStateDiffEq's DynamicSS (abstol 1e-8, reltol 1e-6, tspan Inf) and a tight Newton."""
    import fvmgpu as F

    with pytest.raises(TypeError):
        F.SteadyFVMProblem(object())
    d = F.DynamicSS(F.TRBDF2())
    assert (d.abstol, d.reltol, d.tspan) == (1e-8, 1e-6, float("inf"))
    assert isinstance(d.alg, F.TRBDF2)
    n = F.NewtonRaphson()
    assert (n.abstol, n.reltol, n.max_iters) == (1e-10, 1e-10, 50)
