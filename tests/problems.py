"""Problems of the reference's tests and documentation, restated once and built both for
the oracle and for the GPU API from the same closures (signatures as in the reference:
conditions a(x, y, t, u, p), diffusion D(x, y, t, u, p), flux q(x, y, t, a, b, g, p),
source S(x, y, t, u, p))."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Callable, Dict, Optional, Tuple

import numpy as np

import fvm_oracle as O
from fvmgpu.meshes import triangulate_annulus, triangulate_disk, triangulate_rectangle


@dataclass
class Spec:
    tri: Any
    bc_fns: Tuple
    bc_types: Tuple[str, ...]
    bc_params: Tuple
    ic_fns: Tuple = ()
    ic_params: Tuple = ()
    dirichlet_nodes: Dict[int, int] = field(default_factory=dict)
    dudt_nodes: Dict[int, int] = field(default_factory=dict)
    D: Optional[Callable] = None
    Dp: Any = None
    flux: Optional[Callable] = None
    fluxp: Any = None
    S: Optional[Callable] = None
    Sp: Any = None
    u0: Any = None
    t0: float = 0.0
    tf: float = 1.0


def _bind(f, p):
    return lambda *a: f(*a, p)


def oracle_problem(s: Spec) -> O.Problem:
    conds = O.Conditions(s.tri, [_bind(f, p) for f, p in zip(s.bc_fns, s.bc_params)], list(s.bc_types),
                         [_bind(f, p) for f, p in zip(s.ic_fns, s.ic_params)], s.dirichlet_nodes, s.dudt_nodes)
    return O.Problem(s.tri, conds,
                     flux=_bind(s.flux, s.fluxp) if s.flux else None,
                     D=_bind(s.D, s.Dp) if s.D else None,
                     source=_bind(s.S, s.Sp) if s.S else None, u0=s.u0, t0=s.t0, tf=s.tf)


def rhs_term_scale(prob: O.Problem, u, t):
    """Per-vertex sum of the magnitudes of the terms fvm_eqs! adds up: for each dual edge
    |q(|alpha|, |beta|, |gamma|) . n| l with alpha, beta, gamma formed from |s_v u_v|, scattered
    to both sides; the same for boundary half edges (|Neumann value| l on Neumann edges);
    divided by V; plus |S| or |Dudt value|.  A floating-point evaluation of the RHS is only
    defined to within ~eps times this scale, so parity bounds use
    ||du - ref|| <= tol (||ref|| + ||scale||)."""
    g = prob.geo
    T = g.triangles
    ua = np.abs(np.asarray(u, dtype=np.float64))
    s = np.abs(g.s)
    a = s[:, 0] * ua[T[:, 0]] + s[:, 1] * ua[T[:, 1]] + s[:, 2] * ua[T[:, 2]]
    b = s[:, 3] * ua[T[:, 0]] + s[:, 4] * ua[T[:, 1]] + s[:, 5] * ua[T[:, 2]]
    c = s[:, 6] * ua[T[:, 0]] + s[:, 7] * ua[T[:, 1]] + s[:, 8] * ua[T[:, 2]]
    acc = np.zeros(prob.tri.num_points)
    for e, (a1, a2) in enumerate(((0, 1), (1, 2), (2, 0))):
        qx, qy = O.call_pointwise(prob.flux, g.mid[:, e, 0], g.mid[:, e, 1], t, a, b, c)
        m = (np.abs(qx * g.nrm[:, e, 0]) + np.abs(qy * g.nrm[:, e, 1])) * g.length[:, e]
        np.add.at(acc, T[:, a1], m)
        np.add.at(acc, T[:, a2], m)
    be = prob.tri.boundary_edges
    if be.size:
        Qi, Qj = O.boundary_fluxes(prob, np.asarray(u, dtype=np.float64) * 0 + ua, t)
        np.add.at(acc, be[:, 0], np.abs(Qi))
        np.add.at(acc, be[:, 1], np.abs(Qj))
    out = acc / np.where(prob.geo.cv_volumes > 0, prob.geo.cv_volumes, 1.0)
    src = O.source_contributions(prob, np.zeros_like(acc), ua, t)
    return np.abs(out) + np.abs(src)


def parity_error(got, ref, scale):
    """||got - ref|| / (||ref|| + ||scale||)."""
    return np.linalg.norm(got - ref) / (np.linalg.norm(ref) + np.linalg.norm(scale))


def api_problem(s: Spec, precision="fp64", mesh=None, tile_vertices=0):
    import fvmgpu as F

    mesh = mesh or F.FVMGeometry(s.tri, tile_vertices=tile_vertices)
    types = tuple(getattr(F, t) for t in s.bc_types)
    BCs = F.BoundaryConditions(mesh, tuple(s.bc_fns), types, parameters=tuple(s.bc_params))
    ICs = F.InternalConditions(tuple(s.ic_fns), dirichlet_nodes=s.dirichlet_nodes, dudt_nodes=s.dudt_nodes,
                               parameters=tuple(s.ic_params)) if (s.ic_fns or s.dirichlet_nodes or s.dudt_nodes) else None
    return F.FVMProblem(mesh, BCs, ICs, diffusion_function=s.D, diffusion_parameters=s.Dp, flux_function=s.flux,
                        flux_parameters=s.fluxp, source_function=s.S, source_parameters=s.Sp, initial_condition=s.u0,
                        initial_time=s.t0, final_time=s.tf, precision=precision)


# ---- README / example_diffusion_problem (test/README.jl:4-15; test_functions.jl:304-317) ----
def readme_diffusion(n=50) -> Spec:
    tri = triangulate_rectangle(0.0, 2.0, 0.0, 2.0, n, n, single_boundary=True)
    u0 = np.where(tri.points[:, 1] <= 1.0, 50.0, 0.0)
    return Spec(tri, (lambda x, y, t, u, p: 0.0 * x,), ("Dirichlet",), (None,),
                D=lambda x, y, t, u, p: 1 / 9 + 0.0 * x, u0=u0, tf=0.5)


# ---- heat convection, Neumann on all four sides (test_functions.jl:336-374) ------------------
def heat_convection(n=200) -> Spec:
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    P = dict(alpha=80e-6, q=10.0, k=237.0, h=25.0, Tinf=10.0)
    bot = lambda x, y, t, T, p: -p["alpha"] * p["q"] / p["k"] + 0.0 * x  # noqa: E731
    right = lambda x, y, t, T, p: 0.0 * x  # noqa: E731
    top = lambda x, y, t, T, p: -p["alpha"] * p["h"] / p["k"] * (p["Tinf"] - T)  # noqa: E731
    left = lambda x, y, t, T, p: 0.0 * x  # noqa: E731
    flux = lambda x, y, t, a, b, g, p: (-p["alpha"] * a, -p["alpha"] * b)  # noqa: E731
    u0 = np.full(tri.num_points, 10.0)
    return Spec(tri, (bot, right, top, left), ("Neumann",) * 4, (P, None, P, None), flux=flux, fluxp=P, u0=u0,
                tf=2000.0)


# ---- mixed conditions on an annulus (the reference's example_tri + example_bc_setup kinds) ------
def mixed_annulus(nr=9, ntheta=48, seed=1) -> Spec:
    tri = triangulate_annulus(0.5, 1.0, nr, ntheta, nsegments=4)
    rng = np.random.default_rng(seed)
    fns = (
        lambda x, y, t, u, p: x * y - p + 0.0 * x,       # 0 Dirichlet
        lambda x, y, t, u, p: u * p - 0.3 * x,           # 1 Dudt (affine in u)
        lambda x, y, t, u, p: x + 0.0 * y,               # 2 Neumann
        lambda x, y, t, u, p: y - x,                     # 3 Constrained (never called)
        lambda x, y, t, u, p: p * (1.5 - u),             # 4 Neumann, Robin type
        lambda x, y, t, u, p: 0.2 + 0.0 * x,             # 5 Dirichlet
        lambda x, y, t, u, p: 0.1 * u * u - y,           # 6 Dudt (quadratic in u)
        lambda x, y, t, u, p: 0.0 * x,                   # 7 Neumann, homogeneous
    )
    types = ("Dirichlet", "Dudt", "Neumann", "Constrained", "Neumann", "Dirichlet", "Dudt", "Neumann")
    params = (0.7, 0.3, None, None, 0.8, None, None, None)
    interior = np.nonzero(np.linalg.norm(tri.points, axis=1) < 0.9)[0]
    interior = interior[np.linalg.norm(tri.points[interior], axis=1) > 0.6]
    dnode, dudtnode = int(interior[3]), int(interior[11])
    ic_fns = (lambda x, y, t, u, p: x + y + p + 0.0 * x, lambda x, y, t, u, p: -0.5 * u + p)
    u0 = rng.standard_normal(tri.num_points)
    return Spec(tri, fns, types, params, ic_fns=ic_fns, ic_params=(0.29, 0.1),
                dirichlet_nodes={dnode: 0}, dudt_nodes={dudtnode: 1},
                D=lambda x, y, t, u, p: 1.0 + x * x + 0.5 * y + 0.0 * u,
                S=lambda x, y, t, u, p: p * u - 0.1 * u * u + x, Sp=0.5, u0=u0, t0=0.0, tf=0.1)


# ---- nonlinear diffusion D(u) (porous-medium-like, polynomial in u) -------------------------
def nonlinear_rect(n=30, seed=2) -> Spec:
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    rng = np.random.default_rng(seed)
    fns = (lambda x, y, t, u, p: 0.0 * x, lambda x, y, t, u, p: 0.1 * u,
           lambda x, y, t, u, p: 1.0 + 0.0 * x, lambda x, y, t, u, p: 0.05 * u * u)
    types = ("Dirichlet", "Neumann", "Dirichlet", "Neumann")
    u0 = 0.5 + 0.2 * rng.random(tri.num_points)
    return Spec(tri, fns, types, (None,) * 4, D=lambda x, y, t, u, p: 1.0 + x + 0.5 * u * u,
                S=lambda x, y, t, u, p: u * (1 - u), u0=u0, tf=0.01)


# ---- DiffusionEquation-style field D(x, y) = 1 + 0.5 sin(2 pi x) sin(2 pi y) -----------------
def sine_diffusion(n=64) -> Spec:
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=True)
    P = tri.points
    u0 = np.exp(-50 * ((P[:, 0] - 0.5) ** 2 + (P[:, 1] - 0.5) ** 2))
    D = lambda x, y, t, u, p: 1 + 0.5 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)  # noqa: E731
    return Spec(tri, (lambda x, y, t, u, p: 0.0 * x,), ("Dirichlet",), (None,), D=D, u0=u0, tf=1e-4)


# ---- a wheel: hub vertices of high degree (slices wider than 16 slots) ----------------------
def wheel_mesh(nspoke=40, nring=3):
    """A hub vertex joined to `nspoke` points of the first ring (degree nspoke), then rings of
    quadrilaterals split into triangles; the outer ring is the boundary."""
    from fvmgpu.meshes import Triangulation

    pts = [(0.0, 0.0)]
    for r in range(1, nring + 1):
        th = 2 * np.pi * np.arange(nspoke) / nspoke + 0.1 * r
        pts += list(zip(r / nring * np.cos(th), r / nring * np.sin(th)))
    ring = lambda r, i: 1 + (r - 1) * nspoke + i % nspoke  # noqa: E731
    tris = [(0, ring(1, i), ring(1, i + 1)) for i in range(nspoke)]
    for r in range(1, nring):
        for i in range(nspoke):
            a, b, c, d = ring(r, i), ring(r, i + 1), ring(r + 1, i), ring(r + 1, i + 1)
            tris += [(a, c, d), (a, d, b)]
    boundary = [ring(nring, i) for i in range(nspoke)] + [ring(nring, 0)]
    return Triangulation(np.array(pts), np.array(tris), [boundary])


def wheel_diffusion(nspoke=40) -> Spec:
    tri = wheel_mesh(nspoke)
    P = tri.points
    u0 = np.cos(2 * P[:, 0]) + P[:, 1]
    return Spec(tri, (lambda x, y, t, u, p: 0.5 * u - x,), ("Neumann",), (None,),
                D=lambda x, y, t, u, p: 1.0 + x * x + 0.0 * u, S=lambda x, y, t, u, p: 0.3 * u + y, u0=u0, tf=0.1)


def disk_poisson_mesh(n_interior=3000, n_boundary=128, seed=0):
    return triangulate_disk(n_interior, n_boundary, seed=seed)


# ---- Gray-Scott tutorial system (docs/src/literate_tutorials/gray_scott_model_turing_patterns_...) ----
def gray_scott_oracle(n=30):
    """The tutorial's FVMSystem for the oracle on an n x n mesh of [-1, 1]^2: zero Neumann on the
    whole boundary, fluxes -eps_c grad u_c (eps = 2e-5, 1e-5), sources b (1 - u) - u v^2 and
    -d v + u v^2 (b = 0.04, d = 0.1), initial bump exp(-80 r^2)."""
    tri = triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, n, n, single_boundary=True)
    bc = lambda x, y, t, u: 0.0 * x  # noqa: E731
    conds = [O.Conditions(tri, [bc], ["Neumann"]) for _ in range(2)]
    fluxes = [lambda x, y, t, a, b, g: (-a[0] * 2e-5, -b[0] * 2e-5), lambda x, y, t, a, b, g: (-a[1] * 1e-5, -b[1] * 1e-5)]
    sources = [lambda x, y, t, u: 0.04 * (1 - u[0]) - u[0] * u[1] ** 2, lambda x, y, t, u: -0.1 * u[1] + u[0] * u[1] ** 2]
    P = tri.points
    r2 = P[:, 0] ** 2 + P[:, 1] ** 2
    u0 = np.stack([1 - np.exp(-80 * r2), np.exp(-80 * r2)])
    return O.System(tri, conds, fluxes, sources, u0=u0, tf=6000.0)


# ---- the benchmarked configurations at full size --------------------------------------------
def c2_diffusion(n=1000) -> Spec:
    """The 1000 x 1000 DiffusionEquation workload in FVMProblem form: triangulate_rectangle(0, 1,
    0, 1, n, n) with its four boundary segments, zero Dirichlet on each, D = 1 + 0.5 sin(2 pi x)
    sin(2 pi y), u0 = exp(-50 ((x - 0.5)^2 + (y - 0.5)^2))."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    P = tri.points
    u0 = np.exp(-50 * ((P[:, 0] - 0.5) ** 2 + (P[:, 1] - 0.5) ** 2))
    D = lambda x, y, t, u, p: 1 + 0.5 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) + 0.0 * u  # noqa: E731
    z = lambda x, y, t, u, p: 0.0 * x  # noqa: E731
    return Spec(tri, (z,) * 4, ("Dirichlet",) * 4, (None,) * 4, D=D, u0=u0, tf=1e-4)


def fourier_logfield(seed, sigma=0.5, modes=16):
    """log D(x, y) = sigma sum_m a_m cos(2 pi k_m . x + phi_m) / sqrt(modes / 2) with a_m ~ N(0, 1),
    k_m integer in [1, 4]^2, phi_m ~ U[0, 2 pi), drawn in that order from default_rng(seed): the
    log-normal diffusivity of the batched workload, as a closure of (x, y)."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(modes)
    k = rng.integers(1, 5, size=(modes, 2))
    ph = rng.uniform(0, 2 * np.pi, modes)

    def logD(x, y):
        x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
        s = np.zeros(np.broadcast(x, y).shape)
        for m in range(modes):
            s = s + a[m] * np.cos(2 * np.pi * (k[m, 0] * x + k[m, 1] * y) + ph[m])
        return sigma * s / np.sqrt(modes / 2)
    return logD


# ---- advection-diffusion (docs/src/literate_tutorials/piecewise_linear_and_natural_neighbour_
# interpolation_for_an_advection_diffusion_equation.jl): q = nu u - D grad u, nu = (0.05, 0),
# D = 0.02, zero Dirichlet, u0 = exp(-(x^2 + y^2) / eps^2) / (eps^2 pi), eps = 1/10.  The tutorial
# refines a 2 x 2 rectangle of [-30, 30]^2 with DelaunayTriangulation's refine!, which has no
# restatement here: a uniform n x n grid of the same square stands in for it.
def advection_diffusion(n=121) -> Spec:
    tri = triangulate_rectangle(-30.0, 30.0, -30.0, 30.0, n, n, single_boundary=True)
    P = tri.points
    eps = 0.1
    u0 = np.exp(-(P[:, 0] ** 2 + P[:, 1] ** 2) / eps ** 2) / (eps ** 2 * np.pi)

    def flux(x, y, t, a, b, g, p):
        u = a * x + b * y + g
        return p["nu"] * u - p["D"] * a, -p["D"] * b
    return Spec(tri, (lambda x, y, t, u, p: 0.0 * x,), ("Dirichlet",), (None,), flux=flux,
                fluxp={"D": 0.02, "nu": 0.05}, u0=u0, tf=250.0)


# ---- diffusion on an annulus with a time-dependent inner Dirichlet value -------------------
# (docs/src/literate_tutorials/diffusion_equation_on_an_annulus.jl:34-67): radii 0.2 and 1,
# q . n = 0 on the outer circle, u = 50 (1 - exp(-t/2)) on the inner one, D = 1, the
# tutorial's three-Gaussian initial condition, final time 2, saveat 0.2.  The tutorial refines
# a Delaunay mesh of the annulus; a polar lattice of the same annulus stands in for it.
def annulus_time_dirichlet(nr=24, ntheta=96) -> Spec:
    tri = triangulate_annulus(0.2, 1.0, nr, ntheta, nsegments=1)
    x, y = tri.points[:, 0], tri.points[:, 1]
    u0 = (10 * np.exp(-25 * ((x + 0.5) ** 2 + (y + 0.5) ** 2)) - 5 * np.exp(-50 * ((x + 0.3) ** 2 + (y + 0.5) ** 2))
          - 10 * np.exp(-45 * ((x - 0.5) ** 2 + (y - 0.5) ** 2)))
    fns = (lambda x, y, t, u, p: 0.0 * x, lambda x, y, t, u, p: 50 * (1 - np.exp(-t / 2)) + 0.0 * x)
    return Spec(tri, fns, ("Neumann", "Dirichlet"), (None, None), D=lambda x, y, t, u, p: 1.0 + 0.0 * x, u0=u0,
                tf=2.0)


# ---- the Brusselator's first component with its coupling replaced by -u --------------------
# (docs/src/literate_tutorials/reaction_diffusion_brusselator_system_of_pdes.jl:60-124): on the
# unit square, q = -grad(u)/4, S = -u, and the tutorial's boundary values for Phi
# (q . n = -exp(-x - t/2)/4 below, exp(-1 - y - t/2)/4 right, -exp(-y - t/2)/4 left,
# u = exp(-1 - x - t/2) on top).  u = exp(-x - y - t/2) solves it exactly.
def brusselator_phi(n=40) -> Spec:
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    P = tri.points
    fns = (lambda x, y, t, u, p: -0.25 * np.exp(-x - t / 2),
           lambda x, y, t, u, p: 0.25 * np.exp(-1 - y - t / 2),
           lambda x, y, t, u, p: np.exp(-1 - x - t / 2),
           lambda x, y, t, u, p: -0.25 * np.exp(-y - t / 2))
    return Spec(tri, fns, ("Neumann", "Neumann", "Dirichlet", "Neumann"), (None,) * 4,
                flux=lambda x, y, t, a, b, g, p: (-a / 4, -b / 4), S=lambda x, y, t, u, p: -u,
                u0=np.exp(-P[:, 0] - P[:, 1]), tf=1.0)


def brusselator_phi_exact(x, y, t):
    return np.exp(-x - y - t / 2)


# ---- every kind of time-dependent value, with polynomial and exponential factors ----------
def time_forms_rect(n=30, seed=3) -> Spec:
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    rng = np.random.default_rng(seed)
    fns = (lambda x, y, t, u, p: (2.0 - t) * x,                       # Dirichlet, linear in t
           lambda x, y, t, u, p: 0.1 * t * y + 0.2 * u,               # Neumann, Robin part + t
           lambda x, y, t, u, p: -0.5 * u + np.exp(0.7 * t) * y,      # Dudt, exponential
           lambda x, y, t, u, p: p + 0.0 * x)                         # Neumann, constant
    return Spec(tri, fns, ("Dirichlet", "Neumann", "Dudt", "Neumann"), (None, None, None, 0.3),
                D=lambda x, y, t, u, p: 1.0 + x + 0.0 * u,
                S=lambda x, y, t, u, p: 0.5 * u + (1 + 0.3 * t + 0.2 * t * t) * np.sin(3 * x),
                u0=rng.random(tri.num_points), t0=0.5, tf=1.5)
