"""Pins the oracle (oracle/fvm_oracle.py) to the reference's own known-answer tests.

Each test restates one check of the reference's test suite (paths relative to the
reference project root).  No numeric golden files ship with the reference; these
known-answer tests are the pins.
"""
import numpy as np
import pytest

import fvm_oracle as O
from problems import heat_convection, mixed_annulus, nonlinear_rect, oracle_problem, readme_diffusion, sine_diffusion
from fvmgpu.meshes import triangulate_annulus, triangulate_rectangle


def isapprox(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


# ---- independent control-volume polygons (test/test_functions.jl:1-34) ---------------------------
def cv_polygons(tri):
    """CV polygon of every vertex from its triangle fan, walked counter-clockwise."""
    P = tri.points
    T = tri.triangles
    fans = [[] for _ in range(tri.num_points)]
    for t, (a, b, c) in enumerate(T):
        fans[a].append((b, c, t))
        fans[b].append((c, a, t))
        fans[c].append((a, b, t))
    bnext = {}
    for (u, v) in tri.boundary_edges:
        bnext[int(u)] = int(v)
    polys = []
    for i in range(tri.num_points):
        if not fans[i]:
            polys.append(None)
            continue
        nxt = {a: (b, t) for a, b, t in fans[i]}
        starts = set(nxt) - {b for _, (b, _) in nxt.items()}
        p = P[i]
        pts = []
        if starts:  # boundary vertex: start at the edge (i, a) with the domain on its left
            a = bnext[i]
            pts.append(p)
            while a in nxt:
                b, t = nxt[a]
                c = (P[i] + P[a] + P[b]) / 3
                pts += [(p + P[a]) / 2, c]
                a = b
            pts.append((p + P[a]) / 2)
        else:
            a0 = next(iter(nxt))
            a = a0
            while True:
                b, t = nxt[a]
                pts += [(p + P[a]) / 2, (P[i] + P[a] + P[b]) / 3]
                a = b
                if a == a0:
                    break
        polys.append(np.array(pts))
    return polys


def shoelace(poly):
    x, y = poly[:, 0], poly[:, 1]
    return 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))


@pytest.mark.parametrize("tri", [triangulate_rectangle(0.0, 2.0, 0.0, 5.0, 12, 19, single_boundary=False),
                                 triangulate_annulus(0.5, 1.0, 6, 40)], ids=["rect12x19", "annulus"])
def test_geometry_against_reference_checks(tri):
    """test/geometry.jl:10-76: CV area = polygon area; shape coefficients reproduce a 3x3
    solve and sum to 1; dual-edge midpoints, normals and lengths."""
    g = O.Geometry(tri.points, tri.triangles)
    for i, poly in enumerate(cv_polygons(tri)):
        assert np.isclose(g.cv_volumes[i], shoelace(poly), rtol=1e-12, atol=0)
    rng = np.random.default_rng(0)
    P = tri.points
    for t, (i, j, k) in enumerate(tri.triangles):
        p, q, r = P[i], P[j], P[k]
        u = rng.random(3)
        M = np.array([[p[0], p[1], 1.0], [q[0], q[1], 1.0], [r[0], r[1], 1.0]])
        abc = np.linalg.solve(M, u)
        s = g.s[t]
        got = np.array([s[0:3] @ u, s[3:6] @ u, s[6:9] @ u])
        assert np.allclose(got, abc, rtol=1e-9, atol=1e-9)
        assert np.isclose(s.sum(), 1.0)
        c = (p + q + r) / 3
        mids = [(p + q) / 2, (q + r) / 2, (r + p) / 2]
        for e, m in enumerate(mids):
            assert np.allclose(g.mid[t, e], (c + m) / 2, rtol=1e-14, atol=1e-15)
            ev = c - m
            assert np.isclose(g.length[t, e], np.linalg.norm(ev), rtol=1e-14)
            assert np.allclose(g.nrm[t, e], np.array([ev[1], -ev[0]]) / np.linalg.norm(ev), rtol=1e-14, atol=1e-15)


def test_shape_function_interpolation():
    """test_functions.jl:376-402: alpha x + beta y + gamma reproduces vertex values."""
    s = readme_diffusion(25)
    prob = oracle_problem(s)
    u = s.u0
    T, P = prob.geo.triangles, prob.tri.points
    a, b, c = O._alpha_beta_gamma(prob.geo.s, u[T[:, 0]], u[T[:, 1]], u[T[:, 2]])
    for v in range(3):
        assert np.allclose(a * P[T[:, v], 0] + b * P[T[:, v], 1] + c, u[T[:, v]], atol=1e-9, rtol=0)
    cx, cy = P[T].mean(axis=1).T
    assert np.allclose(a * cx + b * cy + c, u[T].mean(axis=1))


def test_single_triangle_scatter_signs():
    """test_functions.jl:527-556: du_i = Q3 - Q1, du_j = Q1 - Q2, du_k = Q2 - Q3."""
    s = readme_diffusion(12)
    prob = oracle_problem(s)
    u = np.random.default_rng(3).random(s.tri.num_points)
    Q = O.triangle_fluxes(prob, u, 0.0)
    g = prob.geo
    for t in range(0, g.triangles.shape[0], 7):
        i, j, k = g.triangles[t]
        # flux across each dual edge from the closure, directly (test_get_flux, :404-436)
        p, q, r = prob.tri.points[[i, j, k]]
        c = (p + q + r) / 3
        sv = g.s[t]
        al, be, ga = sv[0:3] @ u[[i, j, k]], sv[3:6] @ u[[i, j, k]], sv[6:9] @ u[[i, j, k]]
        for e, (a1, a2) in enumerate(((p, q), (q, r), (r, p))):
            m = (a1 + a2) / 2
            x, y = (c + m) / 2
            ev = c - m
            L = np.linalg.norm(ev)
            qx, qy = prob.flux(x, y, 0.0, al, be, ga)
            assert np.isclose((qx * ev[1] / L - qy * ev[0] / L) * L, Q[t, e], rtol=1e-12, atol=1e-14)
    du = np.zeros_like(u)
    t = 5
    i, j, k = g.triangles[t]
    q1, q2, q3 = Q[t]
    du[i] += q3 - q1
    du[j] += q1 - q2
    du[k] += q2 - q3
    assert np.isclose(du[i], -(q1 - q3)) and np.isclose(du[j], -(-q1 + q2)) and np.isclose(du[k], -(-q2 + q3))


def test_boundary_flux_quarter_points():
    """test_functions.jl:438-525: boundary half-edge fluxes at m_i = (3p+q)/4, m_j = (p+3q)/4."""
    for spec, is_diff in ((readme_diffusion(25), True), (heat_convection(20), False)):
        prob = oracle_problem(spec)
        u = np.random.default_rng(4).random(spec.tri.num_points)
        Qi, Qj = O.boundary_fluxes(prob, u, 0.0)
        P = spec.tri.points
        for m, (i, j) in enumerate(spec.tri.boundary_edges):
            p, q = P[i], P[j]
            L = np.linalg.norm(p - q)
            n = np.array([q[1] - p[1], -(q[0] - p[0])]) / L
            t = prob.bnd_tri[m]
            T = prob.geo.triangles[t]
            sv = prob.geo.s[t]
            al, be, ga = sv[0:3] @ u[T], sv[3:6] @ u[T], sv[6:9] @ u[T]
            for (x, y), Q in ((((3 * p + q) / 4), Qi[m]), (((p + 3 * q) / 4), Qj[m])):
                if is_diff:
                    qx, qy = prob.flux(x, y, 0.0, al, be, ga)
                    ref = (qx * n[0] + qy * n[1]) * np.linalg.norm(p - (p + q) / 2)
                else:
                    f = prob.conds.functions[prob.neumann_fidx[m]]
                    ref = f(x, y, 0.0, al * x + be * y + ga) * np.linalg.norm(p - (p + q) / 2)
                assert np.isclose(Q, ref, rtol=1e-10, atol=1e-14)


def test_source_contribution():
    """test_functions.jl:558-570: du/V (+S = 0), zero on Dirichlet nodes."""
    spec = readme_diffusion(25)
    prob = oracle_problem(spec)
    du = np.random.default_rng(5).random(spec.tri.num_points)
    out = O.source_contributions(prob, du, spec.u0, 0.0)
    ref = du / prob.geo.cv_volumes
    ref[list(prob.conds.dirichlet_nodes)] = 0.0
    assert np.allclose(out, ref, rtol=1e-15, atol=0)


def independent_dudt(spec, u, t, neumann_fns=None):
    """Per-vertex CV-boundary integral of q.n (test_functions.jl:601-657), built from the CV
    polygons, a 3x3 gradient solve per triangle, and the Neumann functions on boundary
    half edges; returns S - (integral)/V with Dirichlet nodes zero."""
    tri = spec.tri
    P = tri.points
    n = tri.num_points
    flux = spec.flux
    p = spec.fluxp
    if flux is None:
        D = spec.D

        def flux(x, y, tt, a, b, g, pp):
            return (-D(x, y, tt, a * x + b * y + g, spec.Dp) * a, -D(x, y, tt, a * x + b * y + g, spec.Dp) * b)
    integral = np.zeros(n)
    T = tri.triangles
    for t, (a, b, c) in enumerate(T):
        M = np.array([[P[a, 0], P[a, 1], 1.0], [P[b, 0], P[b, 1], 1.0], [P[c, 0], P[c, 1], 1.0]])
        al, be, ga = np.linalg.solve(M, u[[a, b, c]])
        cen = (P[a] + P[b] + P[c]) / 3
        for (v, w1, w2) in ((a, b, c), (b, c, a), (c, a, b)):
            pts = [(P[v] + P[w1]) / 2, cen, (P[v] + P[w2]) / 2]
            for q0, q1 in ((pts[0], pts[1]), (pts[1], pts[2])):
                mid = (q0 + q1) / 2
                L = np.linalg.norm(q1 - q0)
                nx, ny = (q1[1] - q0[1]) / L, (q0[0] - q1[0]) / L
                qx, qy = flux(mid[0], mid[1], t, al, be, ga, p)
                integral[v] += L * (qx * nx + qy * ny)
    # boundary half edges of the CVs
    neu = {}
    for s, nodes in enumerate(tri.boundary_nodes):
        for k in range(len(nodes) - 1):
            neu[(int(nodes[k]), int(nodes[k + 1]))] = s
    for m, (i, j) in enumerate(tri.boundary_edges):
        k = tri.boundary_adjacent[m]
        M = np.array([[P[i, 0], P[i, 1], 1.0], [P[j, 0], P[j, 1], 1.0], [P[k, 0], P[k, 1], 1.0]])
        al, be, ga = np.linalg.solve(M, u[[i, j, k]])
        mij = (P[i] + P[j]) / 2
        for v, q0, q1 in ((i, P[i], mij), (j, mij, P[j])):
            mid = (q0 + q1) / 2
            L = np.linalg.norm(q1 - q0)
            nx, ny = (q1[1] - q0[1]) / L, (q0[0] - q1[0]) / L
            s = neu[(int(i), int(j))]
            if spec.bc_types[s] == "Neumann":
                val = spec.bc_fns[s](mid[0], mid[1], t, al * mid[0] + be * mid[1] + ga, spec.bc_params[s])
            else:
                qx, qy = flux(mid[0], mid[1], t, al, be, ga, p)
                val = qx * nx + qy * ny
            integral[v] += L * val
    V = np.array([shoelace(poly) if poly is not None else 1.0 for poly in cv_polygons(tri)])
    S = np.zeros(n) if spec.S is None else np.array([spec.S(P[i, 0], P[i, 1], t, u[i], spec.Sp) for i in range(n)])
    out = S - integral / V
    for s, nodes in enumerate(tri.boundary_nodes):
        if spec.bc_types[s] == "Dirichlet":
            out[np.asarray(nodes)] = 0.0
    return out


@pytest.mark.parametrize("builder", [lambda: readme_diffusion(25), lambda: heat_convection(30)],
                         ids=["diffusion25", "heat_convection30"])
def test_fvm_eqs_against_cv_integrator(builder):
    """test/equations.jl:13-35,94-104 via test_dudt_val (test_functions.jl:648-657)."""
    spec = builder()
    prob = oracle_problem(spec)
    u = spec.u0 if spec.bc_types[0] == "Dirichlet" else spec.u0 + np.random.default_rng(6).random(spec.tri.num_points)
    ref = independent_dudt(spec, u, 0.0)
    got = O.fvm_eqs(prob, u, 0.0)
    assert isapprox(got, ref, 1e-10)
    got_loop = O.fvm_eqs_loop(prob, u, 0.0)
    assert isapprox(got_loop, got, 1e-14)


def test_corner_point_exact():
    """test/equations.jl:37-92: corner vertex of the 200 x 200 heat-convection problem."""
    spec = heat_convection(200)
    prob = oracle_problem(spec)
    u = spec.u0
    P = spec.tri.points
    i, j, k = 0, 1, 200
    x1, y1 = P[j, 0], P[k, 1]
    A = shoelace(np.array([(0.0, 0.0), (x1 / 2, 0.0), (x1 / 3, y1 / 3), (0.0, y1 / 2)]))
    assert np.isclose(prob.geo.cv_volumes[0], A)
    t, _ = prob.geo.find_triangle(np.array([i]), np.array([j]), np.array([k]))
    sv = prob.geo.s[t[0]]
    abc = (sv[0:3] @ u[[i, j, k]], sv[3:6] @ u[[i, j, k]], sv[6:9] @ u[[i, j, k]])
    assert abc == (0.0, 0.0, 10.0)
    Pm = spec.bc_params[0]
    flux1 = -Pm["alpha"] * Pm["q"] / Pm["k"] * (x1 / 2)
    fl = -(1 / A) * (flux1 + 0.0 + 0.0 + 0.0)
    du = O.fvm_eqs(prob, u, 0.0)
    assert np.isclose(du[0], fl, rtol=1e-12)
    assert np.isclose(independent_dudt(heat_convection(20), heat_convection(20).u0, 0.0)[0],
                      O.fvm_eqs(oracle_problem(heat_convection(20)), heat_convection(20).u0, 0.0)[0], rtol=1e-12)


def test_condition_classification():
    """test_functions.jl:192-302 (test_bc_conditions!, test_bc_ic_conditions!) on the 12 x 19
    rectangle with (Dirichlet, Neumann, Dirichlet, Neumann) and internal Dirichlet nodes
    7 + (i-1) 12, i = 2..18 (1-based) -> function 0 (test_functions.jl:98-139)."""
    tri = triangulate_rectangle(0.0, 2.0, 0.0, 5.0, 12, 19, single_boundary=False)
    types = ["Dirichlet", "Neumann", "Dirichlet", "Neumann"]
    fns = [lambda x, y, t, u: x] * 4
    internal = {6 + (i - 1) * 12: 0 for i in range(2, 19)}
    conds = O.Conditions(tri, fns, types, [lambda x, y, t, u: x + y], internal, {})
    nif = 1
    for (u, v), s in zip(tri.boundary_edges, tri.boundary_segment):
        if types[s] == "Dirichlet":
            assert conds.dirichlet_nodes[u] == s + nif and conds.dirichlet_nodes[v] == s + nif
        elif types[s] == "Neumann":
            assert conds.neumann_edges[(u, v)] == s + nif and (u, v) not in conds.constrained_edges
    bnodes = set(np.concatenate(tri.boundary_nodes).tolist())
    for i, f in internal.items():
        if i not in bnodes:
            assert conds.dirichlet_nodes[i] == f
    # the 0-based corner node nx-1 lies on bottom (Dirichlet) and right (Neumann): Dirichlet
    assert conds.dirichlet_nodes[11] == 0 + nif


def test_tsit5_tableau_order_conditions():
    """The restated Tsitouras (2011) tableau: row sums, order 5 for b, order 4 for bhat."""
    c = O.TSIT5_C
    A = np.zeros((7, 7))
    for i, row in enumerate(O.TSIT5_A):
        A[i, : len(row)] = row
    assert np.allclose(A.sum(axis=1), c, atol=1e-14)

    def conds(b):
        Ac = A @ c
        return [
            (b.sum(), 1), (b @ c, 1 / 2), (b @ c**2, 1 / 3), (b @ Ac, 1 / 6), (b @ c**3, 1 / 4),
            (b @ (c * Ac), 1 / 8), (b @ (A @ c**2), 1 / 12), (b @ (A @ Ac), 1 / 24), (b @ c**4, 1 / 5),
            (b @ (c**2 * Ac), 1 / 10), (b @ Ac**2, 1 / 20), (b @ (c * (A @ c**2)), 1 / 15),
            (b @ (c * (A @ Ac)), 1 / 30), (b @ (A @ c**3), 1 / 20), (b @ (A @ (c * Ac)), 1 / 40),
            (b @ (A @ (A @ c**2)), 1 / 60), (b @ (A @ (A @ Ac)), 1 / 120),
        ]
    for got, want in conds(O.TSIT5_B):
        assert abs(got - want) < 1e-12
    bhat = O.TSIT5_B - O.TSIT5_BT
    for got, want in conds(bhat)[:8]:
        assert abs(got - want) < 1e-12
    assert abs(O.TSIT5_BT.sum()) < 1e-15


def test_tsit5_converges_fifth_order():
    """Fixed-step Tsit5 on u' = -u: global error ratio ~ 2^5 on halving dt."""
    f = lambda u, t: -u  # noqa: E731
    errs = []
    for n in (10, 20, 40):
        u = O.tsit5_fixed(None, np.array([1.0]), 0.0, 1.0 / n, n, rhs=f, dirichlet=False)
        errs.append(abs(u[0] - np.exp(-1.0)))
    assert 25 < errs[0] / errs[1] < 40 and 25 < errs[1] / errs[2] < 40


def test_template_matches_generic_rhs():
    """DiffusionEquation A u + b equals fvm_eqs on rows without conditions
    (the doc test diffusion_equations.jl:438 compares the two solutions)."""
    spec = sine_diffusion(24)
    prob = oracle_problem(spec)
    conds = prob.conds
    A, b, u0 = O.template_diffusion(spec.tri, conds, lambda x, y: spec.D(x, y, 0, 0, None), spec.u0)
    u = np.random.default_rng(7).random(spec.tri.num_points)
    free = prob.code == O.FREE
    assert isapprox((A @ u + b)[free], O.fvm_eqs(prob, u, 0.0)[free], 1e-12)


def test_poisson_exact_solution():
    """docs/src/literate_wyos/poissons_equation.jl:92-116 (rtol 1e-4)."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 100, 100, single_boundary=True)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_poisson(tri, conds, lambda x, y: 1.0 + 0.0 * x,
                              lambda x, y: -np.sin(np.pi * x) * np.sin(np.pi * y))
    u = O.steady_solve(A, b)
    P = tri.points
    exact = np.sin(np.pi * P[:, 0]) * np.sin(np.pi * P[:, 1]) / (2 * np.pi**2)
    assert isapprox(u, exact, 1e-4)


def test_mean_exit_time_disk():
    """Mean exit time of a unit disk with D = 1: T(r) = (1 - r^2)/4 (the closed form behind
    docs/src/literate_wyos/mean_exit_time.jl); checks the MET assembly."""
    from fvmgpu.meshes import triangulate_disk

    tri = triangulate_disk(4000, 160, seed=3)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_mean_exit_time(tri, conds, lambda x, y: 1.0 + 0.0 * x)
    T = O.steady_solve(A, b)
    r2 = (tri.points**2).sum(axis=1)
    assert isapprox(T, (1 - r2) / 4, 2e-3)


def test_nonlinear_and_mixed_oracle_consistency():
    """Vectorised and line-by-line restatements agree on the mixed-condition annulus and the
    nonlinear-diffusion rectangle (Dudt, Constrained, Robin Neumann, internal nodes)."""
    for spec in (mixed_annulus(), nonlinear_rect(12)):
        prob = oracle_problem(spec)
        u = spec.u0
        assert isapprox(O.fvm_eqs(prob, u, 0.3), O.fvm_eqs_loop(prob, u, 0.3), 1e-13)


def test_set_diag_assigns_like_a_dense_matrix():
    """The oracle's A[i, i] = value on a sparse matrix equals the assignment on the dense
    matrix, for rows with and without a stored diagonal entry."""
    from scipy.sparse import random as sprandom

    A = sprandom(60, 60, density=0.1, format="csr", random_state=3)
    A.setdiag(np.where(np.arange(60) % 3 == 0, 0.0, 2.5))
    A.eliminate_zeros()
    idx = np.array([0, 3, 4, 5, 17, 18, 59, 4])
    ref = A.toarray()
    ref[idx, idx] = 1.0
    got = O._set_diag(A, idx, 1.0)
    assert np.array_equal(got.toarray(), ref)


def test_tsit5_continuous_extension_order_conditions():
    """Tsit5's dense output (Tsitouras 2011): at theta = 1 the weights are the step's, and for
    every theta the order-4 conditions of a continuous extension hold,
    sum b = theta, b.c = theta^2/2, b.c^2 = theta^3/3, b.Ac = theta^3/6, b.c^3 = theta^4/4,
    b.(c*Ac) = theta^4/8, b.Ac^2 = theta^4/12, b.AAc = theta^4/24."""
    c = O.TSIT5_C
    A = np.zeros((7, 7))
    for i in range(1, 7):
        for j, a in enumerate(O.TSIT5_A[i]):
            A[i, j] = a
    assert np.max(np.abs(O.tsit5_interp_weights(1.0) - O.TSIT5_B)) <= 1e-14
    assert np.max(np.abs(O.tsit5_interp_weights(0.0))) == 0.0
    for th in np.linspace(0.05, 1.0, 12):
        w = O.tsit5_interp_weights(th)
        conds = [w.sum() - th, w @ c - th ** 2 / 2, w @ c ** 2 - th ** 3 / 3, w @ (A @ c) - th ** 3 / 6,
                 w @ c ** 3 - th ** 4 / 4, w @ (c * (A @ c)) - th ** 4 / 8, w @ (A @ c ** 2) - th ** 4 / 12,
                 w @ (A @ (A @ c)) - th ** 4 / 24]
        assert np.max(np.abs(conds)) <= 1e-14, th


def test_tsit5_dense_output_is_fourth_order():
    """On u' = -u the interpolated values inside one step of size h have error O(h^5): halving
    h divides the error by about 32 (at least 20 here)."""
    f = lambda u, t: -u  # noqa: E731
    errs = []
    for h in (0.2, 0.1):
        k = [f(np.array([1.0]), 0.0)]
        for s_ in range(1, 7):
            y = np.array([1.0])
            for j, a in enumerate(O.TSIT5_A[s_]):
                y = y + h * a * k[j]
            k.append(f(y, 0.0))
        th = 0.4
        errs.append(abs(O.tsit5_interpolate(np.array([1.0]), k, h, th)[0] - np.exp(-th * h)))
    assert errs[0] / errs[1] > 20


def test_oracle_time_dependent_values_converge_to_exact_solution():
    """The oracle's fvm_eqs! and Tsit5 driver with values that depend on t: the Brusselator's
    first component with its coupling replaced by -u (exact solution exp(-x - y - t/2)) on 10 x 10
    and 20 x 20 grids; the error at t = 0.5 falls with h."""
    from problems import brusselator_phi, brusselator_phi_exact, oracle_problem

    errs = []
    for n in (10, 20):
        spec = brusselator_phi(n)
        prob = oracle_problem(spec)
        cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
        ref, st = O.tsit5_solve(lambda u, t: O.fvm_eqs(prob, u, t), spec.u0, 0.0, 0.5, [0.5], abstol=1e-9,
                                reltol=1e-9, callback=cb)
        P = spec.tri.points
        exact = brusselator_phi_exact(P[:, 0], P[:, 1], 0.5)
        errs.append(np.max(np.abs(ref[-1] - exact)) / np.max(exact))
        assert st["nrhs"] == 2 + 6 * (st["naccept"] + st["nreject"]) + st["naccept"]  # k1, initial-dt probe
    assert errs[1] < 0.5 * errs[0] < 5e-3, errs


def test_oracle_system_time_dependent_values_converge_to_exact_solution():
    """The oracle's system restatement with time-dependent boundary values: the Brusselator
    tutorial's problem (exact solution Phi = exp(-x - y - t/2), Psi = exp(x + y + t/2)) on
    8 x 8 and 16 x 16 grids to t = 0.3; the error falls with h."""
    from fvmgpu.meshes import triangulate_rectangle

    errs = []
    for n in (8, 16):
        tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
        phi = [lambda x, y, t, u: -np.exp(-x - t / 2) / 4, lambda x, y, t, u: np.exp(-1 - y - t / 2) / 4,
               lambda x, y, t, u: np.exp(-1 - x - t / 2), lambda x, y, t, u: -np.exp(-y - t / 2) / 4]
        psi = [lambda x, y, t, u: np.exp(x + t / 2), lambda x, y, t, u: -np.exp(1 + y + t / 2) / 4,
               lambda x, y, t, u: -np.exp(1 + x + t / 2) / 4, lambda x, y, t, u: np.exp(y + t / 2)]
        conds = [O.Conditions(tri, phi, ["Neumann", "Neumann", "Dirichlet", "Neumann"]),
                 O.Conditions(tri, psi, ["Dirichlet", "Neumann", "Neumann", "Dirichlet"])]
        fluxes = [lambda x, y, t, a, b, g: (-a[0] / 4, -b[0] / 4), lambda x, y, t, a, b, g: (-a[1] / 4, -b[1] / 4)]
        sources = [lambda x, y, t, u: u[0] ** 2 * u[1] - 2 * u[0], lambda x, y, t, u: -u[0] ** 2 * u[1] + u[0]]
        P = tri.points
        u0 = np.stack([np.exp(-P[:, 0] - P[:, 1]), np.exp(P[:, 0] + P[:, 1])])
        sysm = O.System(tri, conds, fluxes, sources, u0=u0, tf=0.3)
        ref, _ = O.tsit5_solve(lambda v, t: O.system_fvm_eqs(sysm, v, t), u0, 0.0, 0.3, [0.3], abstol=1e-10,
                               reltol=1e-10, callback=lambda v, t: O.system_update_dirichlet_nodes(sysm, v, t))
        ex = np.stack([np.exp(-P[:, 0] - P[:, 1] - 0.15), np.exp(P[:, 0] + P[:, 1] + 0.15)])
        errs.append(max(np.max(np.abs(ref[-1][c] - ex[c])) / np.max(ex[c]) for c in range(2)))
    assert errs[1] < 0.5 * errs[0] < 1e-2, errs


def test_oracle_trbdf2_is_second_order():
    """The oracle's TR-BDF2 with fixed steps on a linear problem: halving dt divides the error
    at t = 0.05 (against a tight Tsit5 solution) by about 4."""
    from problems import oracle_problem, sine_diffusion

    spec = sine_diffusion(12)
    prob = oracle_problem(spec)
    f = lambda u, t: O.fvm_eqs(prob, u, t)  # noqa: E731
    ent, n = O.jacobian_sparsity(spec.tri)
    J = O.colored_jacobian(f, spec.u0, 0.0, ent, n, affine=True)
    cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
    ref, _ = O.tsit5_solve(f, spec.u0, 0.0, 0.05, [0.05], abstol=1e-12, reltol=1e-12, callback=cb)
    errs = []
    for dt in (5e-3, 2.5e-3, 1.25e-3):
        sol, st = O.trbdf2_solve(f, lambda u, t: J, spec.u0, 0.0, 0.05, [0.05], dt=dt, adaptive=False,
                                 callback=cb, affine=True)
        errs.append(np.max(np.abs(sol[-1] - ref[-1])))
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 3.5 < r1 < 4.5 and 3.5 < r2 < 4.5, (errs, r1, r2)


def _steady_oracle_problem(tri, bc_fns, bc_types, D=None, S=None, dirichlet_nodes=None):
    conds = O.Conditions(tri, list(bc_fns), list(bc_types), [lambda x, y, t, u: 0.0 * x] if dirichlet_nodes else [],
                         dirichlet_nodes or {})
    prob = O.Problem(tri, conds, D=D, source=S, u0=np.zeros(tri.num_points), t0=0.0, tf=np.inf)
    f = lambda u, t: O.fvm_eqs(prob, u, t)  # noqa: E731
    ent, n = O.jacobian_sparsity(tri)
    jac = lambda u, t: O.colored_jacobian(f, u, t, ent, n)  # noqa: E731
    cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
    return prob, f, jac, cb, O.fixed_rows(tri, [conds])


def test_oracle_steady_newton_reproduces_a_linear_solution():
    """The steady state of the Laplace tutorial's boundary values (0, 100y, 100, 100y on a
    rectangle) without its internal line is u = 100y, which the vertex-centred scheme reproduces
    exactly: the oracle's Newton steady solve returns it to rounding."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 21, 21, single_boundary=False)
    bcs = (lambda x, y, t, u: 0.0 * x, lambda x, y, t, u: 100 * y, lambda x, y, t, u: 100.0 + 0.0 * x,
           lambda x, y, t, u: 100 * y)
    _, f, jac, cb, fixed = _steady_oracle_problem(tri, bcs, ["Dirichlet"] * 4, D=lambda x, y, t, u: 1.0 + 0.0 * x)
    u, it, res = O.steady_newton(f, jac, np.zeros(tri.num_points), 0.0, fixed, callback=cb)
    assert np.max(np.abs(u - 100 * tri.points[:, 1])) <= 1e-9 * 100
    assert it <= 2 and res <= 1e-6


def test_oracle_steady_newton_mean_exit_time_disk():
    """du/dt = div grad u + 1 with u = 0 on the unit disk's boundary: the steady state is the mean
    exit time (1 - r^2)/4, and it matches the oracle's MeanExitTimeProblem assembly solved
    directly."""
    from fvmgpu.meshes import triangulate_disk

    tri = triangulate_disk(1500, 96, seed=3)
    _, f, jac, cb, fixed = _steady_oracle_problem(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"],
                                                  D=lambda x, y, t, u: 1.0 + 0.0 * x,
                                                  S=lambda x, y, t, u: 1.0 + 0.0 * x)
    u, it, _ = O.steady_newton(f, jac, np.zeros(tri.num_points), 0.0, fixed, callback=cb)
    r2 = (tri.points**2).sum(axis=1)
    assert isapprox(u, (1 - r2) / 4, 5e-3)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_mean_exit_time(tri, conds, lambda x, y: 1.0 + 0.0 * x)
    T = O.steady_solve(A, b)
    assert np.max(np.abs(u - T)) <= 1e-9 * np.max(np.abs(T))


def test_oracle_steady_newton_nonlinear_converges_to_the_kirchhoff_solution():
    """div((1 + u^2) grad u) = 0 on the unit square with u + u^3/3 = x + y on the boundary: the
    Kirchhoff transform w = u + u^3/3 is harmonic, so the exact steady state solves
    u + u^3/3 = x + y.  The oracle's Newton steady solve (per-triangle nonlinear fluxes, a
    coloured finite-difference Jacobian at every iteration) converges to it at second order."""

    def exact(x, y):
        w = x + y  # the real root of u^3/3 + u - w = 0 (Cardano)
        s = np.sqrt(9 * w * w / 4 + 1)
        return np.cbrt(1.5 * w + s) + np.cbrt(1.5 * w - s)

    errs = []
    for n in (9, 17, 33):
        tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=True)
        _, f, jac, cb, fixed = _steady_oracle_problem(tri, [lambda x, y, t, u: exact(x, y)], ["Dirichlet"],
                                                      D=lambda x, y, t, u: 1.0 + u * u)
        u, it, res = O.steady_newton(f, jac, np.zeros(tri.num_points), 0.0, fixed, callback=cb)
        assert 2 <= it <= 12 and res <= 1e-8
        errs.append(np.max(np.abs(u - exact(tri.points[:, 0], tri.points[:, 1]))))
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 3.0 < r1 < 5.0 and 3.0 < r2 < 5.0, (errs, r1, r2)


def test_oracle_system_steady_newton_reproduces_a_linear_solution():
    """Two components with constant cross-diffusion, q_u = -(grad u + grad v / 2) and
    q_v = -(grad u / 4 + grad v), sources v - (x - y) and u^2 - (x + y)^2, and Dirichlet values
    u = x + y, v = x - y: the steady state is u = x + y, v = x - y (linear, so every flux is exact,
    and both sources vanish there).  The oracle's system Newton steady solve from zero recovers
    it to rounding."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 15, 15, single_boundary=True)
    conds = [O.Conditions(tri, [lambda x, y, t, u: x + y], ["Dirichlet"]),
             O.Conditions(tri, [lambda x, y, t, u: x - y], ["Dirichlet"])]
    fluxes = [lambda x, y, t, a, b, g: (-(a[0] + a[1] / 2), -(b[0] + b[1] / 2)),
              lambda x, y, t, a, b, g: (-(a[0] / 4 + a[1]), -(b[0] / 4 + b[1]))]
    sources = [lambda x, y, t, u: u[1] - (x - y), lambda x, y, t, u: u[0] * u[0] - (x + y) ** 2]
    N, n = 2, tri.num_points
    sys_ = O.System(tri, conds, fluxes, sources, u0=np.zeros((N, n)), t0=0.0, tf=np.inf)
    f = lambda x, t: O.system_fvm_eqs(sys_, x.reshape(-1, N).T, t).T.ravel()  # noqa: E731
    ent, nn = O.jacobian_sparsity(tri, N)
    jac = lambda x, t: O.colored_jacobian(f, x, t, ent, nn)  # noqa: E731
    cb = lambda x, t: O.system_update_dirichlet_nodes(sys_, x.reshape(-1, N).T, t).T.ravel()  # noqa: E731
    u, it, res = O.steady_newton(f, jac, np.zeros(N * n), 0.0, O.fixed_rows(tri, conds), callback=cb)
    P = tri.points
    want = np.stack([P[:, 0] + P[:, 1], P[:, 0] - P[:, 1]], axis=1).ravel()
    assert np.max(np.abs(u - want)) <= 1e-9 and it >= 2
