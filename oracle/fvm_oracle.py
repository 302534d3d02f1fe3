"""CPU oracle for the vertex-centred finite-volume hot path (TEST INFRASTRUCTURE).

This module is the checker, never the product: only `tests/`,
`__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` may import it.
It restates, in numpy, the reference's CPU algorithm (FiniteVolumeMethod.jl
1.2.3); every function cites the file:line it follows.  Paths are relative to
the reference project root.

Parity status: pinned by the reference's own known-answer tests, restated in
tests/test_oracle_pins.py (control-volume areas against polygon areas,
shape-function identities, dual-edge geometry, single-triangle scatter signs,
boundary quarter-point fluxes, source finalisation, the independent per-vertex
control-volume integrator of test/test_functions.jl:601-657 and the exact
corner-point test of test/equations.jl:37-92).  The Tsit5 stepper follows the
published Tsitouras (2011) tableau; its agreement with OrdinaryDiffEq itself is
unpinned (no reference test fixes Tsit5 numerics).

Indices are 0-based.  Closures keep the reference signatures:
flux `q(x, y, t, alpha, beta, gamma, p) -> (qx, qy)`, diffusion
`D(x, y, t, u, p)`, source `S(x, y, t, u, p)`, condition `a(x, y, t, u, p)`
(parameters are bound by the caller, so the oracle calls `f(x, y, t, u)`).
Closures are called with numpy arrays when they accept them, else per point.
"""
from __future__ import annotations

import numpy as np

FREE, DIRICHLET, DUDT, NOT_A_VERTEX = 0, 1, 2, 3
NEUMANN_T, DUDT_T, DIRICHLET_T, CONSTRAINED_T = "Neumann", "Dudt", "Dirichlet", "Constrained"


# --------------------------------------------------------------------------------------
# closure evaluation helper
# --------------------------------------------------------------------------------------
def call_pointwise(f, *args):
    """Evaluate closure f at broadcast array arguments; per-point fallback."""
    arrs = [np.asarray(a, dtype=np.float64) if a is not None else None for a in args]
    shape = np.broadcast_shapes(*[a.shape for a in arrs if a is not None])
    try:
        with np.errstate(all="ignore"):
            out = f(*[a if a is None else a for a in arrs])
        if isinstance(out, tuple):
            res = tuple(np.broadcast_to(np.asarray(o, dtype=np.float64), shape).copy() for o in out)
            return res
        out = np.asarray(out, dtype=np.float64)
        return np.broadcast_to(out, shape).copy()
    except (ValueError, TypeError):
        pass
    bargs = [None if a is None else np.broadcast_to(a, shape).ravel() for a in arrs]
    n = int(np.prod(shape)) if shape else 1
    first = f(*[None if a is None else float(a[0]) for a in bargs])
    if isinstance(first, tuple):
        outs = [np.empty(n) for _ in first]
        for m in range(n):
            r = f(*[None if a is None else float(a[m]) for a in bargs])
            for c in range(len(outs)):
                outs[c][m] = r[c]
        return tuple(o.reshape(shape) for o in outs)
    out = np.empty(n)
    for m in range(n):
        out[m] = f(*[None if a is None else float(a[m]) for a in bargs])
    return out.reshape(shape)


# --------------------------------------------------------------------------------------
# geometry: src/geometry.jl:99-169
# --------------------------------------------------------------------------------------
class Geometry:
    """FVMGeometry restated (src/geometry.jl:99-169).

    Attributes
    ----------
    cv_volumes : (npoints,)
    s : (ntri, 9) shape-function coefficients s1..s9 (geometry.jl:137-147)
    mid : (ntri, 3, 2) dual-edge midpoints (m_e + c)/2 (geometry.jl:149-151)
    nrm : (ntri, 3, 2) unit normals (e_y, -e_x)/l with e = c - m_e (:153-161)
    length : (ntri, 3) dual-edge lengths
    """

    def __init__(self, points, triangles):
        P = np.asarray(points, dtype=np.float64)
        T = np.asarray(triangles, dtype=np.int64)
        self.points, self.triangles = P, T
        i, j, k = T[:, 0], T[:, 1], T[:, 2]
        px, py = P[i, 0], P[i, 1]
        qx, qy = P[j, 0], P[j, 1]
        rx, ry = P[k, 0], P[k, 1]
        # DelaunayTriangulation statistics: centroid (p+q+r)/3, edge midpoints (p+q)/2, (q+r)/2, (r+p)/2
        cx, cy = (px + qx + rx) / 3, (py + qy + ry) / 3
        m1x, m1y = (px + qx) / 2, (py + qy) / 2
        m2x, m2y = (qx + rx) / 2, (qy + ry) / 2
        m3x, m3y = (rx + px) / 2, (ry + py) / 2
        pcx, pcy = cx - px, cy - py
        qcx, qcy = cx - qx, cy - qy
        rcx, rcy = cx - rx, cy - ry
        m13x, m13y = m1x - m3x, m1y - m3y
        m21x, m21y = m2x - m1x, m2y - m1y
        m32x, m32y = m3x - m2x, m3y - m2y
        S1 = 1 / 2 * np.abs(pcx * m13y - pcy * m13x)
        S2 = 1 / 2 * np.abs(qcx * m21y - qcy * m21x)
        S3 = 1 / 2 * np.abs(rcx * m32y - rcy * m32x)
        vol = np.zeros(P.shape[0])
        # geometry.jl:133-135 accumulates triangle by triangle
        stacked_idx = np.stack([i, j, k], axis=1).ravel()
        stacked_val = np.stack([S1, S2, S3], axis=1).ravel()
        np.add.at(vol, stacked_idx, stacked_val)
        self.cv_volumes = vol
        D = qx * ry - qy * rx - px * ry + rx * py + px * qy - qx * py
        s = np.empty((T.shape[0], 9))
        s[:, 0] = (qy - ry) / D
        s[:, 1] = (ry - py) / D
        s[:, 2] = (py - qy) / D
        s[:, 3] = (rx - qx) / D
        s[:, 4] = (px - rx) / D
        s[:, 5] = (qx - px) / D
        s[:, 6] = (qx * ry - rx * qy) / D
        s[:, 7] = (rx * py - px * ry) / D
        s[:, 8] = (px * qy - qx * py) / D
        self.s = s
        mid = np.empty((T.shape[0], 3, 2))
        mid[:, 0, 0], mid[:, 0, 1] = (m1x + cx) / 2, (m1y + cy) / 2
        mid[:, 1, 0], mid[:, 1, 1] = (m2x + cx) / 2, (m2y + cy) / 2
        mid[:, 2, 0], mid[:, 2, 1] = (m3x + cx) / 2, (m3y + cy) / 2
        self.mid = mid
        nrm = np.empty((T.shape[0], 3, 2))
        length = np.empty((T.shape[0], 3))
        for e, (mx, my) in enumerate(((m1x, m1y), (m2x, m2y), (m3x, m3y))):
            ex, ey = cx - mx, cy - my
            l = np.sqrt(ex * ex + ey * ey)  # LinearAlgebra.norm of a 2-tuple
            length[:, e] = l
            nrm[:, e, 0], nrm[:, e, 1] = ey / l, -ex / l
        self.nrm, self.length = nrm, length
        # key lookup for _safe_get_triangle_props (src/utils.jl:1-11)
        n = max(P.shape[0], 1)
        self._key = {}
        keys = i * n * n + j * n + k
        self._keys_sorted = np.argsort(keys)
        self._keys = keys[self._keys_sorted]
        self._n = n

    def find_triangle(self, a, b, c):
        """Index and rotation of triangle (a,b,c) as stored (utils.jl:1-11).

        Tries (a,b,c), (b,c,a), (c,a,b) in that order, like
        `_safe_get_triangle_props`.  Vectorised over arrays.
        """
        a, b, c = (np.asarray(x, dtype=np.int64) for x in (a, b, c))
        n = self._n
        out = np.full(a.shape, -1, dtype=np.int64)
        rot = np.zeros(a.shape, dtype=np.int64)
        for r, (x, y, z) in enumerate(((a, b, c), (b, c, a), (c, a, b))):
            q = x * n * n + y * n + z
            pos = np.searchsorted(self._keys, q)
            pos = np.minimum(pos, self._keys.size - 1)
            hit = (self._keys[pos] == q) & (out < 0)
            out[hit] = self._keys_sorted[pos[hit]]
            rot[hit] = r
        if np.any(out < 0):
            raise KeyError("triangle not found in geometry")
        return out, rot


def boundary_cv_components(points, i, j):
    """get_boundary_cv_components (src/equations/control_volumes.jl:41-56)."""
    P = points
    px, py = P[i, 0], P[i, 1]
    qx, qy = P[j, 0], P[j, 1]
    lij = np.sqrt((qx - px) ** 2 + (qy - py) ** 2)
    nx, ny = (qy - py) / lij, -(qx - px) / lij
    mijx, mijy = (px + qx) / 2, (py + qy) / 2
    mix, miy = (px + mijx) / 2, (py + mijy) / 2
    mjx, mjy = (qx + mijx) / 2, (qy + mijy) / 2
    li = np.sqrt((mijx - px) ** 2 + (mijy - py) ** 2)
    return nx, ny, mix, miy, mjx, mjy, li


# --------------------------------------------------------------------------------------
# conditions: src/conditions.jl:486-552
# --------------------------------------------------------------------------------------
class Conditions:
    """Conditions restated (src/conditions.jl:310-324, 486-552).

    `functions` = internal functions first, then one per boundary segment
    (conditions.jl:499,518).  Segments are visited in increasing order; the
    reference visits them in the iteration order of DelaunayTriangulation's
    ghost-vertex Dict, which only matters for a node shared by two Dirichlet
    (or two Dudt) segments with different functions (the last visit wins).
    """

    def __init__(self, tri, bc_functions, bc_types, ic_functions=(), dirichlet_nodes=None, dudt_nodes=None):
        if len(bc_functions) != tri.num_ghost_vertices:
            raise AssertionError("The number of boundary conditions must be the same as the number of parts of the mesh's boundary.")
        nif = len(ic_functions)
        self.functions = tuple(ic_functions) + tuple(bc_functions)
        self.neumann_edges = {}
        self.constrained_edges = {}
        self.dirichlet_nodes = dict(dirichlet_nodes or {})
        self.dudt_nodes = dict(dudt_nodes or {})
        for s, nodes in enumerate(tri.boundary_nodes):
            cond = bc_types[s]
            fidx = s + nif
            for a in range(len(nodes) - 1):
                u, v = int(nodes[a]), int(nodes[a + 1])
                if cond == NEUMANN_T:
                    self.neumann_edges[(u, v)] = fidx
                elif cond == CONSTRAINED_T:
                    self.constrained_edges[(u, v)] = fidx
                elif cond == DIRICHLET_T:
                    self.dirichlet_nodes[u] = fidx
                    self.dirichlet_nodes[v] = fidx
                else:
                    self.dudt_nodes[u] = fidx
                    self.dudt_nodes[v] = fidx

    def has_condition(self, i):
        return i in self.dudt_nodes or i in self.dirichlet_nodes

    def vertex_tables(self, npoints, has_vertex):
        """Per-point code and function index, the classification the kernels consume.

        code: NOT_A_VERTEX if the point is in no solid triangle
        (source_contributions.jl:36-37), else DIRICHLET if a Dirichlet node,
        else DUDT if a Dudt node (Dirichlet takes precedence:
        source_contributions.jl:7-11), else FREE.
        """
        code = np.zeros(npoints, dtype=np.int8)
        fidx = np.full(npoints, -1, dtype=np.int32)
        for i, f in self.dudt_nodes.items():
            code[i], fidx[i] = DUDT, f
        for i, f in self.dirichlet_nodes.items():
            code[i], fidx[i] = DIRICHLET, f
        code[~has_vertex] = NOT_A_VERTEX
        fidx[~has_vertex] = -1
        return code, fidx

    def edge_tables(self, boundary_edges):
        """Per boundary edge: Neumann function index or -1 (boundary_edge_contributions.jl:6)."""
        out = np.full(boundary_edges.shape[0], -1, dtype=np.int32)
        for m, (u, v) in enumerate(boundary_edges):
            out[m] = self.neumann_edges.get((int(u), int(v)), -1)
        return out


# --------------------------------------------------------------------------------------
# problem
# --------------------------------------------------------------------------------------
def diffusion_flux(D):
    """construct_flux_function (src/problem.jl:425-440)."""

    def q(x, y, t, a, b, g):
        u = a * x + b * y + g
        Dval = D(x, y, t, u)
        return (-Dval * a, -Dval * b)

    return q


class Problem:
    """FVMProblem restated (src/problem.jl:96-163); closures take (x,y,t,u)."""

    def __init__(self, tri, conds, flux=None, D=None, source=None, u0=None, t0=0.0, tf=1.0):
        self.tri = tri
        self.geo = Geometry(tri.points, tri.triangles)
        self.conds = conds
        self.flux = flux if flux is not None else diffusion_flux(D)
        self.source = source if source is not None else (lambda x, y, t, u: 0.0 * u)
        self.u0 = None if u0 is None else np.asarray(u0, dtype=np.float64)
        self.t0, self.tf = t0, tf
        self.has_vertex = tri.has_vertex()
        self.code, self.fidx = conds.vertex_tables(tri.num_points, self.has_vertex)
        self.neumann_fidx = conds.edge_tables(tri.boundary_edges)
        # boundary edge -> stored triangle (src/equations/boundary_edge_contributions.jl:79-81)
        be = tri.boundary_edges
        self.bnd_tri, self.bnd_rot = self.geo.find_triangle(be[:, 0], be[:, 1], tri.boundary_adjacent)


def _alpha_beta_gamma(s, ui, uj, uk):
    """get_shape_function_coefficients (src/equations/shape_functions.jl:2-9)."""
    a = s[:, 0] * ui + s[:, 1] * uj + s[:, 2] * uk
    b = s[:, 3] * ui + s[:, 4] * uj + s[:, 5] * uk
    g = s[:, 6] * ui + s[:, 7] * uj + s[:, 8] * uk
    return a, b, g


def triangle_fluxes(prob, u, t):
    """Per-triangle Q_e = (q(x_e) . n_e) l_e, e = 1..3 (triangle_contributions.jl:2-7,
    individual_flux_contributions.jl:2-6,27-33, control_volumes.jl:16-21)."""
    g = prob.geo
    T = g.triangles
    a, b, c = _alpha_beta_gamma(g.s, u[T[:, 0]], u[T[:, 1]], u[T[:, 2]])
    Q = np.empty((T.shape[0], 3))
    for e in range(3):
        x, y = g.mid[:, e, 0], g.mid[:, e, 1]
        qx, qy = call_pointwise(prob.flux, x, y, t, a, b, c)
        qn = qx * g.nrm[:, e, 0] + qy * g.nrm[:, e, 1]
        Q[:, e] = qn * g.length[:, e]
    return Q


def boundary_fluxes(prob, u, t):
    """Per boundary edge (Q_i, Q_j) (boundary_edge_contributions.jl:2-13,41-48,77-86)."""
    tri, g = prob.tri, prob.geo
    be = tri.boundary_edges
    i, j = be[:, 0], be[:, 1]
    Tk = g.triangles[prob.bnd_tri]
    a, b, c = _alpha_beta_gamma(g.s[prob.bnd_tri], u[Tk[:, 0]], u[Tk[:, 1]], u[Tk[:, 2]])
    nx, ny, mix, miy, mjx, mjy, l = boundary_cv_components(tri.points, i, j)
    out = []
    for mx, my in ((mix, miy), (mjx, mjy)):
        um = a * mx + b * my + c
        qx, qy = call_pointwise(prob.flux, mx, my, t, a, b, c)
        qn = qx * nx + qy * ny
        neu = prob.neumann_fidx >= 0
        for f in np.unique(prob.neumann_fidx[neu]):
            sel = prob.neumann_fidx == f
            qn[sel] = call_pointwise(prob.conds.functions[f], mx[sel], my[sel], t, um[sel])
        out.append(qn * l)
    return out[0], out[1]


def fvm_eqs(prob, u, t):
    """serial_fvm_eqs! (src/equations/main_equations.jl:38-44).

    Vectorised over entities; the scatter order (np.add.at, in entity order)
    matches a serial loop's order of contributions per vertex, though each
    triangle's pair (Q3 - Q1) is formed before it is added.
    """
    u = np.asarray(u, dtype=np.float64)
    n = u.shape[0]
    du = np.zeros(n)
    T = prob.geo.triangles
    Q = triangle_fluxes(prob, u, t)
    # update_du! (triangle_contributions.jl:10-15)
    idx = np.stack([T[:, 0], T[:, 1], T[:, 2]], axis=1).ravel()
    val = np.stack([Q[:, 2] - Q[:, 0], Q[:, 0] - Q[:, 1], Q[:, 1] - Q[:, 2]], axis=1).ravel()
    np.add.at(du, idx, val)
    # boundary edges (boundary_edge_contributions.jl:61-65)
    Qi, Qj = boundary_fluxes(prob, u, t)
    be = prob.tri.boundary_edges
    np.add.at(du, np.stack([be[:, 0], be[:, 1]], axis=1).ravel(), -np.stack([Qi, Qj], axis=1).ravel())
    return source_contributions(prob, du, u, t)


def source_contributions(prob, du, u, t):
    """get_source_contributions! (src/equations/source_contributions.jl:2-14,33-47,71-76)."""
    P = prob.tri.points
    code, fidx = prob.code, prob.fidx
    out = du.copy()
    free = code == FREE
    if np.any(free):
        S = call_pointwise(prob.source, P[free, 0], P[free, 1], t, u[free])
        out[free] = du[free] / prob.geo.cv_volumes[free] + S
    out[code == DIRICHLET] = 0.0
    out[code == NOT_A_VERTEX] = 0.0
    dd = code == DUDT
    for f in np.unique(fidx[dd]):
        sel = dd & (fidx == f)
        out[sel] = call_pointwise(prob.conds.functions[f], P[sel, 0], P[sel, 1], t, u[sel])
    return out


def fvm_eqs_loop(prob, u, t):
    """Line-by-line serial restatement (main_equations.jl:38-44) for small meshes."""
    g, tri = prob.geo, prob.tri
    du = np.zeros(u.shape[0])
    for m, (i, j, k) in enumerate(g.triangles):
        s = g.s[m]
        a = s[0] * u[i] + s[1] * u[j] + s[2] * u[k]
        b = s[3] * u[i] + s[4] * u[j] + s[5] * u[k]
        c = s[6] * u[i] + s[7] * u[j] + s[8] * u[k]
        Q = []
        for e in range(3):
            x, y = g.mid[m, e]
            qx, qy = prob.flux(x, y, t, a, b, c)
            Q.append((qx * g.nrm[m, e, 0] + qy * g.nrm[m, e, 1]) * g.length[m, e])
        du[i] = du[i] + Q[2] - Q[0]
        du[j] = du[j] + Q[0] - Q[1]
        du[k] = du[k] + Q[1] - Q[2]
    for m, (i, j) in enumerate(tri.boundary_edges):
        tm = prob.bnd_tri[m]
        ti, tj, tk = g.triangles[tm]
        s = g.s[tm]
        a = s[0] * u[ti] + s[1] * u[tj] + s[2] * u[tk]
        b = s[3] * u[ti] + s[4] * u[tj] + s[5] * u[tk]
        c = s[6] * u[ti] + s[7] * u[tj] + s[8] * u[tk]
        nx, ny, mix, miy, mjx, mjy, l = boundary_cv_components(tri.points, i, j)
        qs = []
        for mx, my in ((mix, miy), (mjx, mjy)):
            if prob.neumann_fidx[m] >= 0:
                qn = prob.conds.functions[prob.neumann_fidx[m]](mx, my, t, a * mx + b * my + c)
            else:
                qx, qy = prob.flux(mx, my, t, a, b, c)
                qn = qx * nx + qy * ny
            qs.append(qn * l)
        du[i] = du[i] - qs[0]
        du[j] = du[j] - qs[1]
    out = du.copy()
    for i in range(u.shape[0]):
        x, y = tri.points[i]
        cde = prob.code[i]
        if cde == NOT_A_VERTEX:
            out[i] = 0.0
        elif cde == FREE:
            out[i] = du[i] / g.cv_volumes[i] + prob.source(x, y, t, u[i])
        elif cde == DIRICHLET:
            out[i] = 0.0
        else:
            out[i] = prob.conds.functions[prob.fidx[i]](x, y, t, u[i])
    return out


def update_dirichlet_nodes(prob, u, t):
    """update_dirichlet_nodes! (src/equations/dirichlet.jl:2-8,20-26,38-43)."""
    u = u.copy()
    P = prob.tri.points
    for f in set(prob.conds.dirichlet_nodes.values()):
        nodes = np.array([i for i, g in prob.conds.dirichlet_nodes.items() if g == f], dtype=np.int64)
        u[nodes] = call_pointwise(prob.conds.functions[f], P[nodes, 0], P[nodes, 1], t, u[nodes])
    return u


# --------------------------------------------------------------------------------------
# systems of equations: FVMSystem (src/problem.jl:190-365) and the system branches of
# src/equations/*.jl.  State u is (N, npoints): u[var, i] is component var at node i.
# --------------------------------------------------------------------------------------
def call_system(f, x, y, t, *tuples):
    """Evaluate a system closure f(x, y, t, T1, T2, ...) whose Ti are N-tuples of arrays (the
    reference passes tuples for alpha, beta, gamma and u at quarter points, and the column
    u[:, i] for sources and conditions).  Falls back to one call per point, with tuples of
    floats, when the closure does not accept arrays.  Returns an array, or a tuple of arrays
    for a tuple-valued closure (fluxes)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    T = [tuple(np.broadcast_to(np.asarray(c, dtype=np.float64), (n,)) for c in tup) for tup in tuples]
    try:
        with np.errstate(all="ignore"):
            out = f(x, np.broadcast_to(np.asarray(y, dtype=np.float64), (n,)), t, *T)
        if isinstance(out, tuple):
            return tuple(np.broadcast_to(np.asarray(o, dtype=np.float64), (n,)).copy() for o in out)
        return np.broadcast_to(np.asarray(out, dtype=np.float64), (n,)).copy()
    except (ValueError, TypeError, IndexError):
        pass
    yb = np.broadcast_to(np.asarray(y, dtype=np.float64), (n,))
    res = None
    for m in range(n):
        r = f(float(x[m]), float(yb[m]), t, *[tuple(float(c[m]) for c in tup) for tup in T])
        if res is None:
            res = [np.empty(n) for _ in r] if isinstance(r, tuple) else np.empty(n)
        if isinstance(r, tuple):
            for c, v in enumerate(r):
                res[c][m] = v
        else:
            res[m] = r
    return tuple(res) if isinstance(res, list) else res


class System:
    """FVMSystem(prob1, ..., probN) restated (src/problem.jl:233-365).

    Each component keeps its own conditions (merge_problem_conditions, :336-365: the
    function list of component var is its problem's own, offset by cnum_fncs), flux function
    q_var(x, y, t, alpha, beta, gamma) with N-tuples alpha, beta, gamma, and source
    S_var(x, y, t, u) with u the N-tuple of the node's component values."""

    def __init__(self, tri, conds, fluxes, sources=None, u0=None, t0=0.0, tf=1.0):
        self.N = len(conds)
        if not (len(fluxes) == self.N and (sources is None or len(sources) == self.N)):
            raise AssertionError("one flux and one source per component")
        self.tri = tri
        self.geo = Geometry(tri.points, tri.triangles)
        self.conds = list(conds)
        self.fluxes = list(fluxes)
        zero = lambda x, y, t, u: 0.0 * x  # noqa: E731
        self.sources = [zero if s is None else s for s in (sources or [None] * self.N)]
        self.u0 = None if u0 is None else np.asarray(u0, dtype=np.float64)
        self.t0, self.tf = t0, tf
        self.has_vertex = tri.has_vertex()
        tabs = [c.vertex_tables(tri.num_points, self.has_vertex) for c in self.conds]
        self.code = np.stack([c for c, _ in tabs])
        self.fidx = np.stack([f for _, f in tabs])
        self.neumann_fidx = np.stack([c.edge_tables(tri.boundary_edges) for c in self.conds])
        be = tri.boundary_edges
        self.bnd_tri, self.bnd_rot = self.geo.find_triangle(be[:, 0], be[:, 1], tri.boundary_adjacent)


def _system_abg(s, u, i, j, k):
    """get_shape_function_coefficients for a system (src/equations/shape_functions.jl:12-19)."""
    N = u.shape[0]
    a = tuple(s[:, 0] * u[l, i] + s[:, 1] * u[l, j] + s[:, 2] * u[l, k] for l in range(N))
    b = tuple(s[:, 3] * u[l, i] + s[:, 4] * u[l, j] + s[:, 5] * u[l, k] for l in range(N))
    g = tuple(s[:, 6] * u[l, i] + s[:, 7] * u[l, j] + s[:, 8] * u[l, k] for l in range(N))
    return a, b, g


def system_fvm_eqs(sys, u, t):
    """serial_fvm_eqs! on an FVMSystem (src/equations/main_equations.jl:38-44) with the system
    methods of each part:
    triangles: get_flux for a system (individual_flux_contributions.jl:35-51) and update_du!
    (triangle_contributions.jl:18-25); boundary edges: get_boundary_fluxes and
    _get_boundary_fluxes for a system (boundary_edge_contributions.jl:15-39,50-59,67-75);
    sources: get_source_contribution and fvm_eqs_single_source_contribution! for a system
    (source_contributions.jl:17-30,49-66).  u and the result are (N, npoints)."""
    u = np.asarray(u, dtype=np.float64)
    N, n = u.shape
    g, tri = sys.geo, sys.tri
    T = g.triangles
    du = np.zeros((N, n))
    a, b, c = _system_abg(g.s, u, T[:, 0], T[:, 1], T[:, 2])
    Q = np.empty((N, T.shape[0], 3))
    for e in range(3):
        x, y = g.mid[:, e, 0], g.mid[:, e, 1]
        for var in range(N):
            qx, qy = call_system(sys.fluxes[var], x, y, t, a, b, c)
            Q[var, :, e] = (qx * g.nrm[:, e, 0] + qy * g.nrm[:, e, 1]) * g.length[:, e]
    idx = np.stack([T[:, 0], T[:, 1], T[:, 2]], axis=1).ravel()
    for var in range(N):
        q = Q[var]
        np.add.at(du[var], idx, np.stack([q[:, 2] - q[:, 0], q[:, 0] - q[:, 1], q[:, 1] - q[:, 2]], axis=1).ravel())
    be = tri.boundary_edges
    if be.shape[0]:
        i, j = be[:, 0], be[:, 1]
        Tk = T[sys.bnd_tri]
        a, b, c = _system_abg(g.s[sys.bnd_tri], u, Tk[:, 0], Tk[:, 1], Tk[:, 2])
        nx, ny, mix, miy, mjx, mjy, l = boundary_cv_components(tri.points, i, j)
        for side, (mx, my) in enumerate(((mix, miy), (mjx, mjy))):
            ushape = tuple(a[v] * mx + b[v] * my + c[v] for v in range(N))
            for var in range(N):
                qx, qy = call_system(sys.fluxes[var], mx, my, t, a, b, c)
                qn = (qx * nx + qy * ny) * l
                nf = sys.neumann_fidx[var]
                for f in np.unique(nf[nf >= 0]):
                    sel = nf == f
                    qn[sel] = call_system(sys.conds[var].functions[f], mx[sel], my[sel], t,
                                          tuple(us[sel] for us in ushape)) * l[sel]
                np.add.at(du[var], be[:, side], -qn)
    P = tri.points
    out = du.copy()
    ucols = tuple(u[v] for v in range(N))
    for var in range(N):
        code, fidx = sys.code[var], sys.fidx[var]
        free = code == FREE
        if np.any(free):
            S = call_system(sys.sources[var], P[free, 0], P[free, 1], t, tuple(uc[free] for uc in ucols))
            out[var, free] = du[var, free] / g.cv_volumes[free] + S
        out[var, (code == DIRICHLET) | (code == NOT_A_VERTEX)] = 0.0
        dd = code == DUDT
        for f in np.unique(fidx[dd]):
            sel = dd & (fidx == f)
            out[var, sel] = call_system(sys.conds[var].functions[f], P[sel, 0], P[sel, 1], t,
                                        tuple(uc[sel] for uc in ucols))
    return out


def system_update_dirichlet_nodes(sys, u, t):
    """serial_update_dirichlet_nodes! for a system (src/equations/dirichlet.jl:11-18,28-35,54-61):
    component by component, in place, each node's value from its condition at the node's
    current column u[:, i] (so a later component sees the earlier components' new values)."""
    u = np.array(u, dtype=np.float64)
    P = sys.tri.points
    for var in range(sys.N):
        dn = sys.conds[var].dirichlet_nodes
        for f in set(dn.values()):
            nodes = np.array([i for i, g in dn.items() if g == f], dtype=np.int64)
            u[var, nodes] = call_system(sys.conds[var].functions[f], P[nodes, 0], P[nodes, 1], t,
                                        tuple(u[v, nodes] for v in range(sys.N)))
    return u


def adjacent(tri, i, j):
    """get_adjacent(tri, i, j): the third vertex of the solid triangle holding the oriented
    edge (i, j), or None for an edge with the outside on its left."""
    if not hasattr(tri, "_oracle_adj"):
        adj = {}
        for a, b, c in np.asarray(tri.triangles).reshape(-1, 3):
            a, b, c = int(a), int(b), int(c)
            adj[(a, b)], adj[(b, c)], adj[(c, a)] = c, a, b
        tri._oracle_adj = adj
    return tri._oracle_adj.get((int(i), int(j)))


def _abg_at(prob, T, u):
    """_safe_get_triangle_props then get_shape_function_coefficients (src/utils.jl:1-11,
    shape_functions.jl:2-19): the stored rotation of T and its alpha, beta, gamma (N-tuples for
    an (N, npoints) u)."""
    g = prob.geo
    idx, _ = g.find_triangle(np.array([T[0]]), np.array([T[1]]), np.array([T[2]]))
    t = int(idx[0])
    a, b, c = (int(v) for v in g.triangles[t])
    s = g.s[t]
    u = np.asarray(u, dtype=np.float64)
    if u.ndim == 2:
        return tuple(tuple(s[3 * m] * u[l, a] + s[3 * m + 1] * u[l, b] + s[3 * m + 2] * u[l, c]
                           for l in range(u.shape[0])) for m in range(3))
    return tuple(s[3 * m] * u[a] + s[3 * m + 1] * u[b] + s[3 * m + 2] * u[c] for m in range(3))


def compute_flux(prob, i, j, u, t):
    """compute_flux(prob, i, j, u, t) (src/problem.jl:458-487) for a Problem or a System."""
    P = prob.tri.points
    px, py = P[i]
    qx, qy = P[j]
    ex, ey = qx - px, qy - py
    l = np.sqrt(ex * ex + ey * ey)
    nx, ny = ey / l, -ex / l
    k = adjacent(prob.tri, j, i)
    if k is None:
        k = adjacent(prob.tri, i, j)
    else:
        i, j = j, i
    a, b, c = _abg_at(prob, (i, j, k), u)
    mx, my = (px + qx) / 2, (py + qy) / 2
    if isinstance(prob, System):
        return tuple(nx * qv[0] + ny * qv[1] for qv in (f(mx, my, t, a, b, c) for f in prob.fluxes))
    qvx, qvy = prob.flux(mx, my, t, a, b, c)
    return nx * qvx + ny * qvy


def pl_interpolate(prob, T, u, x, y):
    """pl_interpolate(prob, T, u, x, y) (src/utils.jl:23-27)."""
    a, b, c = _abg_at(prob, T, u)
    if isinstance(a, tuple):
        return np.array([a[l] * x + b[l] * y + c[l] for l in range(len(a))])
    return a * x + b * y + c


def jacobian_sparsity(tri, N=None):
    """jacobian_sparsity(tri) and jacobian_sparsity(tri, N) (src/solve.jl:60-131), restated as
    the reference's loops: every point index i gets (i, i); a vertex also gets (i, j) for each
    neighbour j (get_neighbours, ghost vertices skipped).  With N components, node i's unknowns
    are i N + l (0-based), and every coupled node pair is a full N x N block.  Returns the set of
    (row, column) pairs and the dimension."""
    n = tri.num_points
    nbrs = [set() for _ in range(n)]
    for a, b, c in np.asarray(tri.triangles).reshape(-1, 3):
        for u, v in ((a, b), (b, c), (c, a)):
            nbrs[int(u)].add(int(v))
            nbrs[int(v)].add(int(u))
    has_vertex = tri.has_vertex()
    K = 1 if N is None else int(N)
    entries = set()
    for i in range(n):
        for l in range(K):
            for j in range(K):
                entries.add((i * K + l, i * K + j))
        if not has_vertex[i]:
            continue
        for j in nbrs[i]:
            for l in range(K):
                for k in range(K):
                    entries.add((i * K + l, j * K + k))
    return entries, n * K


def colored_jacobian(f, u, t, entries, n, affine=False):
    """Sparse Jacobian of f at u on the sparsity pattern `entries` (pairs (row, column), e.g.
    from jacobian_sparsity), by finite differences over a greedy colouring of the columns
    (columns that share no row are perturbed together): for an affine f one forward difference
    with unit steps, exact up to rounding; otherwise central differences with steps
    1e-6 (1 + |u_c|).  Test infrastructure for the implicit stepper.  Returns CSR."""
    import scipy.sparse as sp

    rows_of = [[] for _ in range(n)]
    for r, c in entries:
        rows_of[c].append(r)
    color = np.full(n, -1, dtype=np.int64)
    used_rows = []  # per colour, the rows its columns touch
    for c in range(n):
        rs = rows_of[c]
        for k, taken in enumerate(used_rows):
            if not any(r in taken for r in rs):
                color[c] = k
                taken.update(rs)
                break
        else:
            color[c] = len(used_rows)
            used_rows.append(set(rs))
    u = np.asarray(u, dtype=np.float64)
    rr, cc, vv = [], [], []
    f0 = f(u, t) if affine else None
    for k in range(len(used_rows)):
        cols = np.nonzero(color == k)[0]
        step = np.ones(cols.size) if affine else 1e-6 * (1 + np.abs(u[cols]))
        up = u.copy()
        up[cols] += step
        if affine:
            df = f(up, t) - f0
            scale = np.ones(n)
        else:
            um = u.copy()
            um[cols] -= step
            df = f(up, t) - f(um, t)
            scale = np.full(n, 2.0)
        stepc = np.zeros(n)
        stepc[cols] = step
        for c in cols:
            for r in rows_of[c]:
                rr.append(r)
                cc.append(c)
                vv.append(df[r] / (scale[r] * stepc[c]))
    return sp.csr_matrix((vv, (rr, cc)), shape=(n, n))


def trbdf2_solve(f, jac, u0, t0, tf, saveat, dt=None, adaptive=True, abstol=1e-6, reltol=1e-3, callback=None,
                 affine=False, max_steps=10_000_000):
    """TR-BDF2 (Hosea & Shampine, Appl. Numer. Math. 20, 1996), the implicit method the
    reference's tutorials pass to OrdinaryDiffEq, restated with the library's step control and
    exact sparse solves: gamma = 2 - sqrt 2, d = gamma/2, w = sqrt 2/4, z = h f;
      z_g = h f(u_n + d z_n + d z_g),  z_1 = h f(u_n + w z_n + w z_g + d z_1),
      u_{n+1} = u_n + w z_n + w z_g + d z_1;
    each stage by simplified Newton with W = I - d h J(u_n) (`jac(u, t)` gives J), from the
    predictors z_g = z_n and z_1 = z_g; convergence when the update's weighted RMS is <= 1e-10 or
    the rate estimate theta/(1 - theta) times it is <= 1e-2, at most 10 iterations (an affine f
    takes one); a failed stage retries the step with h/4.  Error estimate
    W^-1 ((1 - sqrt 2)/3 z_n + z_g/3 + (sqrt 2 - 2)/3 z_1), accepted when its weighted RMS
    (abstol + reltol max(|u_n|, |u_{n+1}|)) is <= 1; h <- h min(10, max(0.2, 0.9 err^(-1/3))).
    saveat values inside a step: cubic Hermite of (u_n, f_n), (u_{n+1}, f_{n+1}).  The callback
    (the Dirichlet update) runs after every accepted step; f is evaluated again after it when it
    is the first update or it changed u.  Returns (snapshots, stats)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    sq2 = np.sqrt(2.0)
    gam = 2.0 - sq2
    d = gam / 2.0
    w = sq2 / 4.0
    u = np.array(u0, dtype=np.float64)
    n = u.size
    saveat = list(saveat)
    out, si, t = [], 0, t0
    while si < len(saveat) and saveat[si] == t0:
        out.append(u.copy())
        si += 1
    fn = f(u, t)
    nrhs = 1
    tspan = tf - t0

    def wrms(x, a, b=None):
        sc = abstol + reltol * (np.abs(a) if b is None else np.maximum(np.abs(a), np.abs(b)))
        return np.sqrt(np.sum((x / sc) ** 2) / max(1, n))

    h = dt
    if adaptive and not h:
        d0, d1 = wrms(u, u), wrms(fn, u)
        h = min(1e-6 if (d0 < 1e-5 or d1 < 1e-5) else 0.01 * d0 / d1, tspan)
    naccept = nreject = step = newton = failures = 0
    first_cb = True
    I = sp.identity(n, format="csc")
    while t < tf:
        if step >= max_steps:
            raise RuntimeError("max_steps")
        last = t + h >= tf - 1e-12 * tspan
        hh = tf - t if last else h
        step += 1
        zn = hh * fn
        lu = spl.splu((I - d * hh * jac(u, t)).tocsc())

        def stage(z, base, tt):
            nonlocal nrhs, newton
            prev = 0.0
            for it in range(10):
                newton += 1
                r = hh * f(base + d * z, tt) - z
                nrhs += 1
                x = lu.solve(r)
                z += x
                if affine:
                    return True
                dn = wrms(x, u)
                if not np.isfinite(dn):
                    return False
                if dn <= 1e-10:
                    return True
                if it > 0:
                    theta = dn / prev
                    if theta >= 1.0:
                        return False
                    if theta / (1.0 - theta) * dn <= 1e-2:
                        return True
                prev = dn
            return False

        zg = zn.copy()
        ok = stage(zg, u + d * zn, t + gam * hh)
        if ok:
            base = u + w * zn + w * zg
            z1 = zg.copy()
            ok = stage(z1, base, t + hh)
        if not ok:
            failures += 1
            if not adaptive:
                raise RuntimeError("TRBDF2: Newton did not converge at the fixed dt")
            h = hh / 4
            continue
        un = base + d * z1
        err = 0.0
        if adaptive:
            est = lu.solve((1 - sq2) / 3 * zn + zg / 3 + (sq2 - 2) / 3 * z1)
            err = wrms(est, u, un)
            if err > 1.0:
                nreject += 1
                h = hh * min(10.0, max(0.2, 0.9 * err ** (-1.0 / 3.0)))
                continue
        tn = tf if last else t + hh
        f1 = f(un, tn)
        nrhs += 1
        while si < len(saveat) and saveat[si] < tn:
            th = (saveat[si] - t) / hh
            t2, t3 = th * th, th * th * th
            out.append((2 * t3 - 3 * t2 + 1) * u + (t3 - 2 * t2 + th) * hh * fn + (-2 * t3 + 3 * t2) * un
                       + (t3 - t2) * hh * f1)
            si += 1
        u, fn, t = un, f1, tn
        naccept += 1
        if callback is not None:
            ucb = callback(u, t)
            changed = not np.array_equal(ucb, u)
            u = ucb
            if first_cb or changed:
                fn = f(u, t)
                nrhs += 1
            first_cb = False
        while si < len(saveat) and saveat[si] == t:
            out.append(u.copy())
            si += 1
        if adaptive:
            q = 0.9 * err ** (-1.0 / 3.0) if err > 0 else 10.0
            h = min(tspan, hh * min(10.0, max(0.2, q)))
        if last:
            break
    while si < len(saveat):
        out.append(u.copy())
        si += 1
    return np.array(out), {"naccept": naccept, "nreject": nreject, "nrhs": nrhs, "newton": newton,
                           "failures": failures}


def fixed_rows(tri, conds_list):
    """The rows a steady solve holds at their values, over states flattened [point][component]:
    a component's Dirichlet nodes and every point in no triangle (du/dt = 0 there, and the
    Jacobian row is zero).  Test infrastructure for the steady solvers."""
    N = len(conds_list)
    fixed = np.zeros((tri.num_points, N))
    hv = tri.has_vertex()
    for r, c in enumerate(conds_list):
        fixed[list(c.dirichlet_nodes.keys()), r] = 1.0
        fixed[~hv, r] = 1.0
    return fixed.ravel()


def steady_newton(f, jac, u0, t, fixed, abstol=1e-10, reltol=1e-10, max_iters=50, callback=None):
    """A steady state of du/dt = f(u, t) (SteadyFVMProblem, src/problem.jl:166-180, solved with
    NonlinearSolve's NewtonRaphson, src/solve.jl:184-196), restated with exact sparse solves:
    the Dirichlet update at t (`callback`) on the guess, then u <- u + du with
    (F - J(u)) du = f(u), F = diag(fixed) (the fixed rows keep their values, where J's rows
    vanish), until max|f(u)| <= abstol or <= reltol max|f(u) + u|.  Test infrastructure.
    Returns (u, Newton iterations, max|f(u)|)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    u = np.array(u0, dtype=np.float64)
    if callback is not None:
        u = callback(u, t)
    F = sp.diags(np.asarray(fixed, dtype=np.float64))
    for it in range(max_iters + 1):
        r = f(u, t)
        res = float(np.max(np.abs(r)))
        if res <= abstol or res <= reltol * float(np.max(np.abs(r + u))):
            return u, it, res
        if it == max_iters:
            break
        u = u + spl.spsolve((F - jac(u, t)).tocsc(), r)
    raise RuntimeError("steady_newton did not converge")


# --------------------------------------------------------------------------------------
# linear templates: src/specific_problems/*.jl, assembled sparse (not dense)
# --------------------------------------------------------------------------------------
def _template_A_entries(tri, geo, conds, D, rows, cols, vals):
    """triangle_contributions! (src/specific_problems/abstract_templates.jl:73-99)."""
    T = geo.triangles
    V = geo.cv_volumes
    hc = np.zeros(tri.num_points, dtype=bool)
    for d in (conds.dirichlet_nodes, conds.dudt_nodes):
        hc[list(d.keys())] = True
    s = geo.s
    for e, (a1, a2) in enumerate(((0, 1), (1, 2), (2, 0))):
        x, y = geo.mid[:, e, 0], geo.mid[:, e, 1]
        nx, ny = geo.nrm[:, e, 0], geo.nrm[:, e, 1]
        Dl = call_pointwise(D, x, y) * geo.length[:, e]
        e1, e2 = T[:, a1], T[:, a2]
        for vert in range(3):
            a = Dl * (s[:, vert] * nx + s[:, 3 + vert] * ny)
            m1 = ~hc[e1]
            rows.append(e1[m1]); cols.append(T[m1, vert]); vals.append(a[m1] / V[e1[m1]])
            m2 = ~hc[e2]
            rows.append(e2[m2]); cols.append(T[m2, vert]); vals.append(-a[m2] / V[e2[m2]])
    return hc


def _template_boundary(tri, geo, conds, D, hc, rows, cols, vals, b, with_neumann=True):
    """boundary_edge_contributions! (abstract_templates.jl:149-191,237-267).

    Reproduces the reference's use of V_i for row j in the non-Neumann part
    (abstract_templates.jl:262)."""
    V = geo.cv_volumes
    be = tri.boundary_edges
    tidx, _ = geo.find_triangle(be[:, 0], be[:, 1], tri.boundary_adjacent)
    for m, (i, j) in enumerate(be):
        i, j = int(i), int(j)
        nx, ny, mix, miy, mjx, mjy, l = boundary_cv_components(tri.points, i, j)
        Di = float(call_pointwise(D, mix, miy))
        Dj = float(call_pointwise(D, mjx, mjy))
        if (i, j) in conds.neumann_edges:
            if not with_neumann:
                continue
            f = conds.functions[conds.neumann_edges[(i, j)]]
            ai = float(np.asarray(f(mix, miy, None, None)))
            aj = float(np.asarray(f(mjx, mjy, None, None)))
            if not conds.has_condition(i):
                b[i] += Di * ai * l / V[i]
            if not conds.has_condition(j):
                b[j] += Dj * aj * l / V[j]
            continue
        tm = tidx[m]
        ijk = geo.triangles[tm]
        s = geo.s[tm]
        for vert in range(3):
            w = s[vert] * nx + s[3 + vert] * ny
            if not hc[i]:
                rows.append(np.array([i])); cols.append(np.array([ijk[vert]])); vals.append(np.array([Di * l * w / V[i]]))
            if not hc[j]:
                rows.append(np.array([j])); cols.append(np.array([ijk[vert]])); vals.append(np.array([Dj * l * w / V[i]]))


def _csr(n, rows, cols, vals):
    from scipy.sparse import coo_matrix

    r = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    c = np.concatenate(cols) if cols else np.zeros(0, np.int64)
    v = np.concatenate(vals) if vals else np.zeros(0)
    A = coo_matrix((v, (r, c)), shape=(n, n)).tocsr()
    A.sum_duplicates()
    return A


def _eval_at_points(f, P, nodes):
    return np.array([float(np.asarray(f(P[i, 0], P[i, 1], None, None))) for i in nodes]) if len(nodes) else np.zeros(0)


def template_diffusion(tri, conds, D, ic, reaction=None):
    """DiffusionEquation / LinearReactionDiffusionEquation assembly
    (diffusion_equation.jl:69-101; linear_reaction_diffusion_equations.jl:76-125).

    Returns (A, b, u0) with du/dt = A u + b; u0 has Dirichlet values applied
    (abstract_templates.jl:109-117)."""
    geo = Geometry(tri.points, tri.triangles)
    n = tri.num_points
    rows, cols, vals = [], [], []
    b = np.zeros(n)
    hc = _template_A_entries(tri, geo, conds, D, rows, cols, vals)
    _template_boundary(tri, geo, conds, D, hc, rows, cols, vals, b)
    if reaction is not None:  # linear_source_contributions! (:115-125)
        free = np.nonzero(~hc & tri.has_vertex())[0]
        rows.append(free); cols.append(free); vals.append(call_pointwise(reaction, tri.points[free, 0], tri.points[free, 1]))
    # apply_dudt_conditions! (abstract_templates.jl:127-135)
    P = tri.points
    for i, f in conds.dudt_nodes.items():
        if i not in conds.dirichlet_nodes:
            b[i] = float(np.asarray(conds.functions[f](P[i, 0], P[i, 1], None, None)))
    u0 = np.array(ic, dtype=np.float64)
    for i, f in conds.dirichlet_nodes.items():
        u0[i] = float(np.asarray(conds.functions[f](P[i, 0], P[i, 1], None, None)))
    # fix_missing_vertices! (:317-325)
    miss = np.nonzero(~tri.has_vertex())[0]
    rows.append(miss); cols.append(miss); vals.append(np.ones(miss.size)); b[miss] = 0.0
    return _csr(n, rows, cols, vals), b, u0


def template_poisson(tri, conds, D, f):
    """PoissonsEquation assembly (poissons_equation.jl:58-88; create_rhs_b
    abstract_templates.jl:278-288; apply_steady_dirichlet_conditions! :302-309)."""
    if conds.dudt_nodes:
        raise ValueError("PoissonsEquation does not support Dudt nodes.")
    geo = Geometry(tri.points, tri.triangles)
    n = tri.num_points
    P = tri.points
    hv = tri.has_vertex()
    b = np.zeros(n)
    nd = np.array([i for i in range(n) if hv[i] and i not in conds.dirichlet_nodes], dtype=np.int64)
    if nd.size:
        b[nd] = call_pointwise(f, P[nd, 0], P[nd, 1])
    rows, cols, vals = [], [], []
    hc = _template_A_entries(tri, geo, conds, D, rows, cols, vals)
    _template_boundary(tri, geo, conds, D, hc, rows, cols, vals, b)
    for i, g in conds.dirichlet_nodes.items():
        b[i] = float(np.asarray(conds.functions[g](P[i, 0], P[i, 1], None, None)))
    dn = np.array(sorted(conds.dirichlet_nodes), dtype=np.int64)
    A = _csr(n, rows, cols, vals)
    A = _set_diag(A, dn, 1.0)
    miss = np.nonzero(~hv)[0]
    A = _set_diag(A, miss, 1.0)
    b[miss] = 0.0
    return A, b


def template_mean_exit_time(tri, conds, D):
    """MeanExitTimeProblem assembly (mean_exit_time.jl:57-94): triangle
    contributions only; b = -1 off Dirichlet nodes, A_ii = 1 on them."""
    if conds.dudt_nodes:
        raise ValueError("MeanExitTimeProblem does not support Dudt nodes.")
    if conds.constrained_edges:
        raise ValueError("MeanExitTimeProblem does not support Constrained edges.")
    geo = Geometry(tri.points, tri.triangles)
    n = tri.num_points
    hv = tri.has_vertex()
    rows, cols, vals = [], [], []
    _template_A_entries(tri, geo, conds, D, rows, cols, vals)
    b = np.zeros(n)
    dmask = np.zeros(n, dtype=bool)
    dmask[list(conds.dirichlet_nodes.keys())] = True
    b[hv & ~dmask] = -1.0
    A = _csr(n, rows, cols, vals)
    A = _set_diag(A, np.nonzero(hv & dmask)[0], 1.0)
    miss = np.nonzero(~hv)[0]
    A = _set_diag(A, miss, 1.0)
    b[miss] = 0.0
    return A, b


def _set_diag(A, idx, value):
    """A[i, i] = value for i in idx (assignment, not accumulation).  Stored diagonal entries of
    those rows are overwritten and missing ones are added, so the result is exactly `value`
    whatever was accumulated there before."""
    from scipy.sparse import coo_matrix

    idx = np.unique(np.asarray(idx, dtype=np.int64))
    if idx.size == 0:
        return A
    M = A.tocoo()
    on = (M.row == M.col) & np.isin(M.row, idx)
    data = M.data.copy()
    data[on] = value
    missing = np.setdiff1d(idx, M.row[on])
    r = np.concatenate([M.row, missing])
    c = np.concatenate([M.col, missing])
    v = np.concatenate([data, np.full(missing.size, float(value))])
    return coo_matrix((v, (r, c)), shape=A.shape).tocsr()


# --------------------------------------------------------------------------------------
# Tsit5 (Tsitouras 2011), restated from the published tableau
# --------------------------------------------------------------------------------------
TSIT5_C = np.array([0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0])
TSIT5_A = [
    [],
    [0.161],
    [-0.008480655492356989, 0.335480655492357],
    [2.897153057105493, -6.359448489975075, 4.3622954328695815],
    [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525],
    [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383],
    [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774],
]
TSIT5_B = np.array(TSIT5_A[6] + [0.0])
# b - bhat (error estimate weights)
TSIT5_BT = np.array([
    -0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
    -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 0.015151515151515152,
])


def tsit5_step(f, u, t, dt, k1=None):
    """One Tsit5 step.  Returns (u_new, k list of 7 stage derivatives)."""
    k = [f(u, t) if k1 is None else k1]
    for s in range(1, 7):
        y = u.copy()
        for j, a in enumerate(TSIT5_A[s]):
            y += dt * a * k[j]
        k.append(f(y, t + TSIT5_C[s] * dt))
    # the 7th stage point equals u_new (FSAL)
    unew = u.copy()
    for j in range(6):
        unew += dt * TSIT5_B[j] * k[j]
    return unew, k


def tsit5_fixed(prob, u0, t0, dt, nsteps, rhs=None, dirichlet=True):
    """Fixed-step Tsit5 with the Dirichlet callback after every step
    (src/solve.jl:133-144: DiscreteCallback with condition true)."""
    f = rhs or (lambda u, t: fvm_eqs(prob, u, t))
    u = np.array(u0, dtype=np.float64)
    t = t0
    k1 = None
    for _ in range(nsteps):
        u, k = tsit5_step(f, u, t, dt, k1)
        t = t0 + (_ + 1) * dt
        if dirichlet and prob is not None and prob.conds.dirichlet_nodes:
            u = update_dirichlet_nodes(prob, u, t)
            k1 = None  # the callback modified u: FSAL derivative re-evaluated
        else:
            k1 = k[6]
    return u


def tsit5_interp_weights(th):
    """Weights b_i(theta) of Tsit5's free 4th-order continuous extension (Tsitouras 2011,
    Comput. Math. Appl. 62:770-775, the dense output OrdinaryDiffEq's Tsit5 interpolates saveat
    with): u(t_n + theta h) = u_n + h sum_i b_i(theta) k_i over the seven stages, k_7 the FSAL
    derivative f(u_{n+1}).  b_i(1) are the step's weights; the order-4 conditions hold for every
    theta (checked in the tests)."""
    t = th
    return np.array([
        -1.0530884977290216 * t * (t - 1.3299890189751412) * (t * t - 1.4364028541716351 * t + 0.7139816917074209),
        0.1017 * t * t * (t * t - 2.1966568338249754 * t + 1.2949852507374631),
        2.490627285651252793 * t * t * (t * t - 2.38535645472061657 * t + 1.57803468208092486),
        -16.54810288924490272 * (t - 1.21712927295533244) * (t - 0.61620406037800089) * t * t,
        47.37952196281928122 * (t - 1.203071208372362603) * (t - 0.658047292653547382) * t * t,
        -34.87065786149660974 * (t - 1.2) * (t - 0.666666666666666667) * t * t,
        2.5 * (t - 1) * (t - 0.6) * t * t])


def tsit5_interpolate(u, k, h, th):
    """u(t_n + theta h) from the step's start u and its seven stage derivatives k."""
    w = tsit5_interp_weights(th)
    acc = w[0] * k[0]
    for j in range(1, 7):
        acc = acc + w[j] * k[j]
    return u + h * acc


def tsit5_solve(f, u0, t0, tf, saveat, dt=None, adaptive=True, abstol=1e-6, reltol=1e-3, callback=None,
                max_steps=10_000_000):
    """Tsit5 driver with the step control of OrdinaryDiffEq's defaults for Tsit5 (PI
    controller beta1 = 7/50, beta2 = 2/25, qmin = 1/5, qmax = 10, gamma = 9/10,
    qoldinit = 1e-4; RMS error norm; Hairer initial step) and a per-step callback applied
    after each accepted step (src/solve.jl:133-144).  saveat values inside a step come from
    Tsit5's own continuous extension of the pre-callback step (tsit5_interpolate); values at a
    step end are the post-callback state.  Returns (snapshots, stats)."""
    u = np.array(u0, dtype=np.float64)
    n = u.size
    saveat = list(saveat)
    out = []
    si = 0
    t = t0
    while si < len(saveat) and saveat[si] == t0:
        out.append(u.copy())
        si += 1
    k1 = f(u, t)
    nrhs = 1
    tspan = tf - t0
    rms = lambda v: np.sqrt(np.sum(v * v) / max(1, n))  # noqa: E731
    if adaptive and not dt:
        sc = abstol + np.abs(u) * reltol
        d0, d1 = rms(u / sc), rms(k1 / sc)
        dt0 = 1e-6 if (d0 < 1e-5 or d1 < 1e-5) else 0.01 * d0 / d1
        dt0 = min(dt0, tspan)
        f1 = f(u + dt0 * k1, t + dt0)
        nrhs += 1
        d2 = rms((f1 - k1) / sc) / dt0
        md = max(d1, d2)
        dt1 = max(1e-6, dt0 * 1e-3) if md <= 1e-15 else 10.0 ** (-(2.0 + np.log10(md)) / 5.0)
        dt = min(100 * dt0, dt1, tspan)
    beta1, beta2, qmin, qmax, gamma = 7 / 50, 2 / 25, 0.2, 10.0, 0.9
    qold = 1e-4
    nfixed = 0 if adaptive else int(np.ceil(tspan / dt - 1e-9))
    step = naccept = nreject = 0
    first_cb = True
    while (t < tf) if adaptive else (step < nfixed):
        if step >= max_steps:
            raise RuntimeError("max_steps")
        if adaptive:
            last = t + dt >= tf
            h = tf - t if last else dt
        else:
            last = step + 1 == nfixed
            tn_ = tf if last else t0 + (step + 1) * dt
            h = tn_ - t
        k = [k1]
        for s_ in range(1, 7):
            y = u.copy()
            for j, a in enumerate(TSIT5_A[s_]):
                y += h * a * k[j]
            if s_ < 6:
                k.append(f(y, t + TSIT5_C[s_] * h))
                nrhs += 1
        unew = y
        k.append(f(unew, t + h))
        nrhs += 1
        if adaptive:
            err = h * sum(TSIT5_BT[j] * k[j] for j in range(7))
            EEst = rms(err / (abstol + np.maximum(np.abs(u), np.abs(unew)) * reltol))
            if EEst == 0:
                q = 1 / qmax
                q11 = 0.0
            else:
                q11 = EEst ** beta1
                q = max(1 / qmax, min(1 / qmin, q11 / qold ** beta2 / gamma))
            if EEst > 1:
                nreject += 1
                step += 1
                dt = h / min(1 / qmin, q11 / gamma)
                continue
        tn = tf if last else (t + h if adaptive else t0 + (step + 1) * dt)
        while si < len(saveat) and saveat[si] < tn:
            out.append(tsit5_interpolate(u, k, h, (saveat[si] - t) / h))
            si += 1
        u = unew
        t = tn
        naccept += 1
        step += 1
        reeval = False
        if callback is not None:
            # OrdinaryDiffEq evaluates the first-same-as-last derivative again after a callback
            # that modifies u; one that rewrites the values u already holds changes nothing
            # (Dirichlet rows have du = 0, so after the first update a time-independent value
            # is already in place and f(u) is the step's last stage)
            ucb = callback(u, t)
            reeval = first_cb or not np.array_equal(ucb, u)
            u = ucb
            first_cb = False
        while si < len(saveat) and saveat[si] == t:
            out.append(u.copy())
            si += 1
        if reeval:
            k1 = f(u, t)
            nrhs += 1
        else:
            k1 = k[6]
        if adaptive:
            qold = max(EEst, 1e-4)
            dt = min(h / q, tspan)
        if last:
            break
    while si < len(saveat):
        out.append(u.copy())
        si += 1
    return np.array(out), {"naccept": naccept, "nreject": nreject, "nrhs": nrhs}


def steady_solve(A, b):
    """Direct sparse solve of A u = b (stands in for LinearSolve's KLU in the docs)."""
    from scipy.sparse.linalg import spsolve

    return spsolve(A.tocsc(), b)


# --------------------------------------------------------------------------------------
# fields given by vertex values (the adjoint's log-diffusivity parametrisation)
# --------------------------------------------------------------------------------------
def p1_field(tri, values):
    """The continuous piecewise-linear interpolant of per-vertex `values` over the solid
    triangles of `tri`, as a closure f(x, y, *ignored) for the template constructors (the
    reference evaluates D(x, y) at dual-edge midpoints and boundary quarter points).  Each
    query point is located by its barycentric coordinates; points on a shared edge get the
    same value from either triangle."""
    P = np.asarray(tri.points, dtype=np.float64)
    T = np.asarray(tri.triangles, dtype=np.int64)
    vals = np.asarray(values, dtype=np.float64)

    def f(x, y, *_):
        shape = np.broadcast(np.asarray(x), np.asarray(y)).shape
        xs, ys = (np.broadcast_to(np.asarray(c, dtype=np.float64), shape).ravel() for c in (x, y))
        out = np.full(xs.shape, np.nan)
        todo = np.ones(xs.shape, dtype=bool)
        for a, b, c in T:
            if not todo.any():
                break
            (ax, ay), (bx, by), (cx, cy) = P[a], P[b], P[c]
            det = (bx - ax) * (cy - ay) - (cx - ax) * (by - ay)
            la = ((bx - xs) * (cy - ys) - (cx - xs) * (by - ys)) / det
            lb = ((cx - xs) * (ay - ys) - (ax - xs) * (cy - ys)) / det
            lc = 1.0 - la - lb
            tol = -1e-12
            hit = todo & (la >= tol) & (lb >= tol) & (lc >= tol)
            out[hit] = la[hit] * vals[a] + lb[hit] * vals[b] + lc[hit] * vals[c]
            todo &= ~hit
        if todo.any():
            raise ValueError("p1_field: a query point lies outside the mesh")
        return out.reshape(shape) if shape else float(out[0])

    return f


def template_ode_solve(A, b, u0, dt, nsteps):
    """Fixed-step Tsit5 on du/dt = A u + b (the templates' ODEProblem, no callback)."""
    return tsit5_fixed(None, u0, 0.0, dt, nsteps, rhs=lambda u, t: A @ u + b, dirichlet=False)
