"""Host mirror of FiniteVolumeMethod.jl's public API for the vertex-centred hot path.

Names, argument meanings and error behaviour follow the reference (FiniteVolumeMethod.jl
1.2.3); indices are 0-based (Python), function indices included.  Every compute call goes
through libfvmgpu.so (include/fvm_gpu.h); there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field
from typing import Any, Callable, Dict, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import (FVM_FP32, FVM_FP64, FVM_VERTEX_DIRICHLET, FVM_VERTEX_DUDT, FVM_VERTEX_FREE,
                   FVM_VERTEX_NOT_A_VERTEX, UnsupportedFormError, as_f64, as_i8, as_i32, check, dptr, load)
from .forms import (classify_flux, classify_linear_flux, classify_system_flux, classify_system_poly, classify_xytu, monomials,
                    sample_xy)
from .meshes import Triangulation


# --------------------------------------------------------------------------------------
# conditions (src/conditions.jl)
# --------------------------------------------------------------------------------------
class ConditionType(enum.Enum):
    """src/conditions.jl:36-41."""

    Neumann = 0
    Dudt = 1
    Dirichlet = 2
    Constrained = 3


Neumann = ConditionType.Neumann
Dudt = ConditionType.Dudt
Dirichlet = ConditionType.Dirichlet
Constrained = ConditionType.Constrained


class ParametrisedFunction:
    """f(args...) = fnc(args..., parameters) (src/conditions.jl:16-20)."""

    __slots__ = ("fnc", "parameters")

    def __init__(self, fnc, parameters=None):
        self.fnc = fnc
        self.parameters = parameters

    def __call__(self, *args):
        return self.fnc(*args, self.parameters)


def _as_tuple(x):
    return tuple(x) if isinstance(x, (tuple, list)) else (x,)


def _functions_and_parameters(functions, parameters):
    """A single function takes `parameters` as its own p (conditions.jl:246-251,262-269);
    a tuple of functions takes a tuple of parameters, one each (default nothing)."""
    if not isinstance(functions, (tuple, list)):
        return (functions,), (parameters,)
    fs = tuple(functions)
    ps = tuple(parameters) if parameters is not None else (None,) * len(fs)
    return fs, ps


class BoundaryConditions:
    """BoundaryConditions(mesh, functions, types; parameters) (src/conditions.jl:164-172,237-251).

    functions[s] and types[s] belong to boundary segment s (ghost vertex -(s+1))."""

    def __init__(self, mesh, functions, types, parameters=None):
        fs, ps = _functions_and_parameters(functions, parameters)
        ts = _as_tuple(types)
        if len(fs) != len(ts):
            raise AssertionError("The number of functions and types must be the same.")
        if not all(isinstance(t, ConditionType) for t in ts):
            raise AssertionError("The condition types must be ConditionType instances.")
        if len(fs) != mesh.triangulation.num_ghost_vertices:
            raise AssertionError("The number of boundary conditions must be the same as the number of parts of the "
                                 "mesh's boundary.")
        if len(ps) != len(fs):
            raise AssertionError("The number of parameters must match the number of functions.")
        self.functions = tuple(ParametrisedFunction(f, p) for f, p in zip(fs, ps))
        self.condition_types = ts

    def __repr__(self):
        n = len(self.functions)
        return f"BoundaryConditions with {n} boundary condition{'s' if n > 1 else ''} with types {self.condition_types}"


class InternalConditions:
    """InternalConditions(functions; dirichlet_nodes, dudt_nodes, parameters)
    (src/conditions.jl:223-230,253-269).  Node -> function index (0-based)."""

    def __init__(self, functions=(), dirichlet_nodes: Optional[Dict[int, int]] = None,
                 dudt_nodes: Optional[Dict[int, int]] = None, parameters=None):
        fs, ps = _functions_and_parameters(functions, parameters)
        if len(ps) != len(fs):
            raise AssertionError("The number of parameters must match the number of functions.")
        self.functions = tuple(ParametrisedFunction(f, p) for f, p in zip(fs, ps))
        self.dirichlet_nodes = dict(dirichlet_nodes or {})
        self.dudt_nodes = dict(dudt_nodes or {})

    def __repr__(self):
        return f"InternalConditions with {len(self.dirichlet_nodes)} Dirichlet nodes and {len(self.dudt_nodes)} Dudt nodes"


class Conditions:
    """Merged conditions (src/conditions.jl:310-324; prepare_conditions :486-504;
    merge_conditions! :506-544).  Internal functions come first, then one function per
    boundary segment.  Segments are merged in increasing segment order, so on a node
    shared by two Dirichlet (or two Dudt) segments the later segment's function wins."""

    def __init__(self, mesh, bc: BoundaryConditions, ic: Optional[InternalConditions] = None):
        ic = ic or InternalConditions()
        tri = mesh.triangulation
        nif = len(ic.functions)
        self.functions = ic.functions + bc.functions
        self.neumann_edges: Dict[Tuple[int, int], int] = {}
        self.constrained_edges: Dict[Tuple[int, int], int] = {}
        self.dirichlet_nodes: Dict[int, int] = dict(ic.dirichlet_nodes)
        self.dudt_nodes: Dict[int, int] = dict(ic.dudt_nodes)
        for s, nodes in enumerate(tri.boundary_nodes):
            ctype = bc.condition_types[s]
            f = s + nif
            for a in range(len(nodes) - 1):
                u, v = int(nodes[a]), int(nodes[a + 1])
                if ctype is Neumann:
                    self.neumann_edges[(u, v)] = f
                elif ctype is Constrained:
                    self.constrained_edges[(u, v)] = f
                elif ctype is Dirichlet:
                    self.dirichlet_nodes[u] = f
                    self.dirichlet_nodes[v] = f
                else:
                    self.dudt_nodes[u] = f
                    self.dudt_nodes[v] = f

    # predicates of src/conditions.jl:342-484
    def is_dirichlet_node(self, i):
        return i in self.dirichlet_nodes

    def is_dudt_node(self, i):
        return i in self.dudt_nodes

    def is_neumann_edge(self, i, j):
        return (i, j) in self.neumann_edges

    def is_constrained_edge(self, i, j):
        return (i, j) in self.constrained_edges

    def has_condition(self, i):
        return i in self.dudt_nodes or i in self.dirichlet_nodes

    def has_dirichlet_nodes(self):
        return bool(self.dirichlet_nodes)

    def has_dudt_nodes(self):
        return bool(self.dudt_nodes)

    def has_neumann_edges(self):
        return bool(self.neumann_edges)

    def has_constrained_edges(self):
        return bool(self.constrained_edges)

    def eval_condition_fnc(self, fidx, x, y, t, u):
        return self.functions[fidx](x, y, t, u)

    def vertex_tables(self, has_vertex: np.ndarray):
        """Per-point FVM_VERTEX_* code and function index (Dirichlet before Dudt:
        source_contributions.jl:5-11)."""
        n = has_vertex.shape[0]
        code = np.zeros(n, dtype=np.int8)
        fidx = np.full(n, -1, dtype=np.int32)
        for i, f in self.dudt_nodes.items():
            code[i], fidx[i] = FVM_VERTEX_DUDT, f
        for i, f in self.dirichlet_nodes.items():
            code[i], fidx[i] = FVM_VERTEX_DIRICHLET, f
        code[~has_vertex] = FVM_VERTEX_NOT_A_VERTEX
        fidx[~has_vertex] = -1
        return code, fidx

    def neumann_table(self, boundary_edges: np.ndarray):
        out = np.full(boundary_edges.shape[0], -1, dtype=np.int32)
        for m, (u, v) in enumerate(boundary_edges):
            out[m] = self.neumann_edges.get((int(u), int(v)), -1)
        return out

    def __repr__(self):
        return (f"Conditions with\n   {len(self.neumann_edges)} Neumann edges\n   {len(self.constrained_edges)} "
                f"Constrained edges\n   {len(self.dirichlet_nodes)} Dirichlet nodes\n   {len(self.dudt_nodes)} Dudt nodes")


# --------------------------------------------------------------------------------------
# geometry (src/geometry.jl)
# --------------------------------------------------------------------------------------
@dataclass(frozen=True)
class TriangleProperties:
    """src/geometry.jl:21-26."""

    shape_function_coefficients: Tuple[float, ...]
    cv_edge_midpoints: Tuple[Tuple[float, float], ...]
    cv_edge_normals: Tuple[Tuple[float, float], ...]
    cv_edge_lengths: Tuple[float, float, float]


class FVMGeometry:
    """FVMGeometry(tri) (src/geometry.jl:44-49,99-169): the mesh flattened once into
    Hilbert-ordered device arrays by libfvmgpu.  `cv_volumes` and `triangle_props` keep the
    reference's meaning (caller numbering).  The geometry, the Hilbert order and the operator
    pattern are computed on the device; host_ingest=True computes them on the host instead
    (the two give identical meshes)."""

    def __init__(self, tri: Triangulation, tile_vertices: int = 0, renumber: bool = True, host_ingest: bool = False):
        lib = load()
        _lib.require_gpu()
        self.triangulation = tri
        pts = as_f64(tri.points)
        tris = as_i32(tri.triangles)
        be = as_i32(tri.boundary_edges)
        badj = as_i32(tri.boundary_adjacent)
        h = C.c_void_p()
        check(lib.fvm_mesh_create(dptr(pts), tri.num_points, dptr(tris, _lib.c_int32_p), tri.num_triangles,
                                  dptr(be, _lib.c_int32_p), dptr(badj, _lib.c_int32_p), tri.num_boundary_edges,
                                  int(tile_vertices), (0 if renumber else _lib.FVM_MESH_NO_RENUMBER)
                                  | (_lib.FVM_MESH_HOST_INGEST if host_ingest else 0), C.byref(h)))
        self._h = h
        self.cv_volumes = np.empty(tri.num_points)
        self._props = np.empty((tri.num_triangles, 24))
        check(lib.fvm_mesh_geometry(h, dptr(self.cv_volumes), dptr(self._props)))
        self._triangle_props = None

    @property
    def handle(self):
        return self._h

    @property
    def props_array(self) -> np.ndarray:
        """(ntri, 24): s1..s9, dual-edge midpoints, unit normals, lengths."""
        return self._props

    @property
    def triangle_props(self) -> Dict[Tuple[int, int, int], TriangleProperties]:
        if self._triangle_props is None:
            d = {}
            for t, (i, j, k) in enumerate(self.triangulation.triangles):
                p = self._props[t]
                d[(int(i), int(j), int(k))] = TriangleProperties(
                    tuple(p[0:9]), tuple(map(tuple, p[9:15].reshape(3, 2))), tuple(map(tuple, p[15:21].reshape(3, 2))),
                    tuple(p[21:24]))
            self._triangle_props = d
        return self._triangle_props

    def sample_points(self):
        """(dual-edge midpoints (ntri, 3, 2), boundary quarter points (nbe, 2, 2))."""
        tri = self.triangulation
        dual = np.empty((tri.num_triangles, 3, 2))
        quarter = np.empty((tri.num_boundary_edges, 2, 2))
        check(load().fvm_mesh_sample_points(self._h, dptr(dual), dptr(quarter)))
        return dual, quarter

    def info(self) -> Dict[str, int]:
        a = np.zeros(10, dtype=np.int64)
        check(load().fvm_mesh_info(self._h, dptr(a, _lib.c_int64_p)))
        keys = ["npoints", "ntri", "nbedge", "nvertices", "ntiles", "ntile_elements", "nbedge_elements",
                "tile_vertices", "operator_slots", "operator_nnz"]
        return dict(zip(keys, (int(v) for v in a)))

    def permutation(self) -> np.ndarray:
        p = np.empty(self.triangulation.num_points, dtype=np.int32)
        check(load().fvm_mesh_permutation(self._h, dptr(p, _lib.c_int32_p)))
        return p

    def locate(self, x, y=None, stream=None):
        """Triangle holding each query point, on the device (fvm_mesh_locate): the caller index
        of a solid triangle containing (x[q], y[q]) (the lowest such index for points on shared
        edges), -1 outside the mesh.  x, y: host arrays (or x an (nq, 2) array and y None), or an
        (nq, 2) CUDA float64 tensor as x; returns int64 of the same kind."""
        xy = _query_points(x, y)
        p, loc = _lib.array_pointer(xy)
        out = _like(xy, (xy.shape[0],), "int64")
        op, _ = _lib.array_pointer(out, "int64")
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_mesh_locate(self._h, xy.shape[0], p, op, loc, s))
        return out

    def export_connectivity(self):
        tri = self.triangulation
        t = np.empty((tri.num_triangles, 3), dtype=np.int32)
        b = np.empty((tri.num_boundary_edges, 3), dtype=np.int32)
        check(load().fvm_mesh_export_connectivity(self._h, dptr(t, _lib.c_int32_p), dptr(b, _lib.c_int32_p)))
        return t, b

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._LIB is not None:
            _lib._LIB.fvm_mesh_destroy(h)
            self._h = None

    def __repr__(self):
        tri = self.triangulation
        return f"FVMGeometry with {int(tri.has_vertex().sum())} control volumes, {tri.num_triangles} triangles"


# --------------------------------------------------------------------------------------
# problem descriptors
# --------------------------------------------------------------------------------------
class _Desc:
    """Owns the numpy arrays behind a ProblemDesc."""

    def __init__(self):
        self.keep = []
        self.c = _lib.ProblemDesc()

    def arr(self, name, a, ctype=_lib.c_double_p):
        if a is None:
            setattr(self.c, name, None)
            return
        self.keep.append(a)
        setattr(self.c, name, a.ctypes.data_as(ctype))


class _TimeParts:
    """The time factors of a problem's values and, per factor, the B arrays of each kind
    (descriptor fields time_factor, time_dirichlet, time_neumann, time_source, time_dudt)."""

    def __init__(self, sizes):
        self.factors = []
        self.sizes = sizes  # kind -> length of one factor's array
        self.values = {kind: [] for kind in sizes}

    def add(self, kind, tau, sel, B):
        for g, f in enumerate(self.factors):
            if f.close_to(tau):
                break
        else:
            if len(self.factors) == _lib.FVM_MAX_TIME_FACTORS:
                raise UnsupportedFormError(_lib.FVM_ERR_UNSUPPORTED_FORM, f"more than {_lib.FVM_MAX_TIME_FACTORS} "
                                           "distinct time factors")
            self.factors.append(tau)
            for kd in self.values:
                self.values[kd].append(None)
            g = len(self.factors) - 1
        if self.values[kind][g] is None:
            self.values[kind][g] = np.zeros(self.sizes[kind])
        self.values[kind][g][sel] += B

    def fill(self, d):
        d.c.ntime = len(self.factors)
        if not self.factors:
            return
        d.arr("time_factor", as_f64(np.array(self.factors, dtype=np.float64)))
        for kind, vals in self.values.items():
            if all(v is None for v in vals):
                d.arr(kind, None)
            else:
                d.arr(kind, as_f64(np.stack([np.zeros(self.sizes[kind]) if v is None else v for v in vals])))


def _group_eval(points_by_entity, fidx_by_entity, functions, t0, what, max_degree, time=None):
    """Classify condition functions per function index over the entities that use them.
    points_by_entity: (n, k, 2); returns coefficients (n, k, deg+1) and deg.  time =
    (tf, _TimeParts, kind) allows a time factor on the constant term, recorded in the parts
    (entities flattened to n * k)."""
    n, k = points_by_entity.shape[:2]
    results = {}
    deg = 0
    for f in np.unique(fidx_by_entity[fidx_by_entity >= 0]):
        sel = fidx_by_entity == f
        P = points_by_entity[sel].reshape(-1, 2)
        name = f"{what} function {int(f)}"
        if time is None:
            c, d = classify_xytu(functions[int(f)], P[:, 0], P[:, 1], t0, name, max_degree)
        else:
            tf, parts, kind = time
            c, d, tp = classify_xytu(functions[int(f)], P[:, 0], P[:, 1], t0, name, max_degree, tf=tf, time=True)
            if tp is not None:
                parts.add(kind, tp[0], np.repeat(sel, k), tp[1])
        results[int(f)] = (sel, c)
        deg = max(deg, d)
    out = np.zeros((n, k, deg + 1))
    for f, (sel, c) in results.items():
        cc = np.zeros((c.shape[0], deg + 1))
        cc[:, : c.shape[1]] = c
        out[sel] = cc.reshape(-1, k, deg + 1)
    return out, deg


def _precision(p):
    if p in (FVM_FP64, "fp64", "float64", np.float64, None):
        return FVM_FP64
    if p in (FVM_FP32, "fp32", "float32", np.float32):
        return FVM_FP32
    raise ValueError(f"unknown precision {p!r}")


class FVMProblem:
    """FVMProblem(mesh, boundary_conditions[, internal_conditions]; ...)
    (src/problem.jl:96-163).  The closures are classified into device-coded forms when the
    problem is first used (`handle`, `fvm_eqs`, `solve`), as the reference evaluates them only
    when it solves; forms outside the device-coded set raise UnsupportedFormError there.  A
    problem that is a component of an FVMSystem is never classified on its own: its closures
    take the tuple of all components.

    precision: "fp64" (default) or "fp32" (FP32 flux assembly with FP64 control-volume
    division; linear forms only)."""

    def __init__(self, mesh: FVMGeometry, boundary_conditions: BoundaryConditions,
                 internal_conditions: Optional[InternalConditions] = None, *, diffusion_function=None,
                 diffusion_parameters=None, source_function=None, source_parameters=None, flux_function=None,
                 flux_parameters=None, initial_condition, initial_time=0.0, final_time, precision="fp64"):
        tri = mesh.triangulation
        ic = np.asarray(initial_condition, dtype=np.float64)
        if ic.shape[0] != tri.num_points:
            raise AssertionError("The initial condition must have the same number of elements as the number of "
                                 "nodes in the mesh (including nodes that aren't vertices in the mesh itself).")
        if flux_function is None and diffusion_function is None:
            raise ValueError("provide a diffusion_function or a flux_function")
        self.mesh = mesh
        self.conditions = Conditions(mesh, boundary_conditions, internal_conditions)
        self.diffusion_function = diffusion_function
        self.diffusion_parameters = diffusion_parameters
        self.flux_function = flux_function
        self.flux_parameters = flux_parameters
        self.source_function = source_function
        self.source_parameters = source_parameters
        self.initial_condition = ic
        self.initial_time = float(initial_time)
        self.final_time = float(final_time)
        self.precision = _precision(precision)
        self._h = None
        self._built = False

    # construct_flux_function (src/problem.jl:425-440) happens through the device form:
    # q = -D(x, y, u(x_sigma)) grad u, D a polynomial of degree <= 2 in u.
    def _build(self):
        mesh, tri, conds = self.mesh, self.mesh.triangulation, self.conditions
        t0 = self.initial_time
        hv = tri.has_vertex()
        code, fidx = conds.vertex_tables(hv)
        neu = conds.neumann_table(tri.boundary_edges)
        dual, quarter = mesh.sample_points()
        d = _Desc()
        tf = self.final_time
        parts = _TimeParts({"time_dirichlet": tri.num_points, "time_neumann": 2 * tri.num_boundary_edges,
                            "time_source": tri.num_points, "time_dudt": tri.num_points})
        self._code, self._fidx, self._neu = code, fidx, neu
        d.arr("vertex_code", as_i8(code), _lib.c_int8_p)
        d.arr("bedge_neumann", as_i8(neu >= 0), _lib.c_int8_p)
        dual_M = quarter_M = None
        if self.flux_function is not None:
            q = ParametrisedFunction(self.flux_function, self.flux_parameters)
            try:  # the diffusion form -D(x, y) grad u
                Dd = classify_flux(q, dual[..., 0].ravel(), dual[..., 1].ravel(), t0)
                Dq = (classify_flux(q, quarter[..., 0].ravel(), quarter[..., 1].ravel(), t0) if tri.num_boundary_edges
                      else np.zeros(0))
                ddeg, dual_c, quarter_c = 0, Dd.reshape(-1, 1), Dq.reshape(-1, 1)
            except UnsupportedFormError:  # else any flux linear in (alpha, beta, gamma), e.g. advection
                dual_M = classify_linear_flux(q, dual[..., 0].ravel(), dual[..., 1].ravel(), t0)
                quarter_M = (classify_linear_flux(q, quarter[..., 0].ravel(), quarter[..., 1].ravel(), t0)
                             if tri.num_boundary_edges else np.zeros((0, 6)))
                ddeg, dual_c, quarter_c = 0, np.zeros((0, 1)), np.zeros((0, 1))
        else:
            Df = ParametrisedFunction(self.diffusion_function, self.diffusion_parameters)
            allp = np.concatenate([dual.reshape(-1, 2), quarter.reshape(-1, 2)])
            c, ddeg = classify_xytu(Df, allp[:, 0], allp[:, 1], t0, "diffusion_function")
            nd = dual.reshape(-1, 2).shape[0]
            dual_c, quarter_c = c[:nd], c[nd:]
        d.c.diffusion_degree = ddeg
        d.arr("dual_edge_D", as_f64(dual_c) if dual_c.size else None)
        d.arr("quarter_D", as_f64(quarter_c) if quarter_c.size else None)
        d.arr("dual_edge_flux", as_f64(dual_M) if dual_M is not None else None)
        d.arr("quarter_flux", as_f64(quarter_M) if quarter_M is not None and quarter_M.size else None)
        # Neumann q.n = a(x, y, t, u) at the quarter points of each Neumann edge
        if np.any(neu >= 0):
            nc, ndeg = _group_eval(quarter, neu, conds.functions, t0, "Neumann", 2, (tf, parts, "time_neumann"))
            d.c.neumann_degree = ndeg
            d.arr("quarter_neumann", as_f64(nc.reshape(-1, ndeg + 1)))
        else:
            d.c.neumann_degree = 0
            d.arr("quarter_neumann", None)
        P = tri.points
        # source on free vertices
        free = code == FVM_VERTEX_FREE
        if self.source_function is not None and np.any(free):
            S = ParametrisedFunction(self.source_function, self.source_parameters)
            c, sdeg, tp = classify_xytu(S, P[free, 0], P[free, 1], t0, "source_function", tf=tf, time=True)
            if tp is not None:
                parts.add("time_source", tp[0], free, tp[1])
            src = np.zeros((tri.num_points, sdeg + 1))
            src[free] = c
            d.c.source_degree = sdeg
            d.arr("source", as_f64(src))
        else:
            d.c.source_degree = 0
            d.arr("source", None)
        # Dudt and Dirichlet values per function group
        pts3 = P.reshape(-1, 1, 2)
        dfidx = np.where(code == FVM_VERTEX_DUDT, fidx, -1)
        if np.any(dfidx >= 0):
            dc, udeg = _group_eval(pts3, dfidx, conds.functions, t0, "Dudt", 2, (tf, parts, "time_dudt"))
            d.c.dudt_degree = udeg
            d.arr("dudt", as_f64(dc.reshape(-1, udeg + 1)))
        else:
            d.c.dudt_degree = 0
            d.arr("dudt", None)
        rfidx = np.where(code == FVM_VERTEX_DIRICHLET, fidx, -1)
        if np.any(rfidx >= 0):
            rc, _ = _group_eval(pts3, rfidx, conds.functions, t0, "Dirichlet", 0, (tf, parts, "time_dirichlet"))
            d.arr("dirichlet", as_f64(rc.reshape(-1)))
        else:
            d.arr("dirichlet", None)
        parts.fill(d)
        self.time_factors = list(parts.factors)
        d.c.precision = self.precision
        h = C.c_void_p()
        check(load().fvm_problem_create(mesh.handle, C.byref(d.c), C.byref(h)))
        self._h = h
        self._desc = d
        self.diffusion_degree = ddeg

    @property
    def handle(self):
        if not self._built:
            self._build()
            self._built = True
        return self._h

    def info(self) -> Dict[str, int]:
        a = np.zeros(6, dtype=np.int64)
        check(load().fvm_problem_info(self.handle, dptr(a, _lib.c_int64_p)))
        keys = ["linear", "operator_nonzeros", "operator_slots", "has_constant", "has_quadratic", "precision"]
        return dict(zip(keys, (int(v) for v in a)))

    def export_codes(self):
        tri = self.mesh.triangulation
        code = np.empty(tri.num_points, dtype=np.int8)
        neu = np.empty(tri.num_boundary_edges, dtype=np.int8)
        check(load().fvm_problem_export_codes(self.handle, dptr(code, _lib.c_int8_p), dptr(neu, _lib.c_int8_p)))
        return code, neu

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._LIB is not None:
            _lib._LIB.fvm_problem_destroy(h)
            self._h = None

    def __repr__(self):
        return (f"FVMProblem with {int(self.mesh.triangulation.has_vertex().sum())} nodes and time span "
                f"({self.initial_time}, {self.final_time})")


def _prob_of(p):
    if isinstance(p, (FVMProblem, _Template, FVMSystem)):
        return p
    if isinstance(p, dict):
        return p["prob"]
    return getattr(p, "prob")


def fvm_eqs(du, u, p, t, *, force_triangle=False, conservative=False, internal=False, stream=None):
    """fvm_eqs!(du, u, p, t) (src/equations/main_equations.jl:28-81).  `p` is the problem or
    any object / dict with a `prob` entry.  du, u: float64 numpy arrays (host) or CUDA torch
    tensors (device), caller numbering; internal=True takes device tensors already in the
    library's internal (Hilbert) numbering, as a device-resident time loop holds them.
    Returns du."""
    prob = _prob_of(p)
    if isinstance(prob, _Template):
        return prob.apply(du, u, stream=stream)
    if isinstance(prob, FVMSystem):
        return prob.rhs(du, u, t, internal=internal, stream=stream)
    up, ul = _lib.array_pointer(u)
    dp, dl = _lib.array_pointer(du)
    if ul != dl:
        raise TypeError("u and du must both be host arrays or both device tensors")
    if internal:
        if ul != _lib.FVM_PTR_DEVICE:
            raise TypeError("internal=True needs device tensors")
        ul = _lib.FVM_PTR_DEVICE_INTERNAL
    flags = ul | (_lib.FVM_RHS_FORCE_TRIANGLE if force_triangle else 0) | (
        _lib.FVM_RHS_CONSERVATIVE if conservative else 0)
    s = stream if stream is not None else _lib.current_stream_handle()
    check(load().fvm_rhs(prob.handle, up, dp, float(t), flags, s))
    return du


def update_dirichlet_nodes(u, prob, t=0.0, stream=None):
    """update_dirichlet_nodes! (src/equations/dirichlet.jl:78-86), in place."""
    prob = _prob_of(prob)
    if isinstance(prob, FVMSystem):
        return prob.update_dirichlet_nodes(u, t, stream)
    up, ul = _lib.array_pointer(u)
    s = stream if stream is not None else _lib.current_stream_handle()
    check(load().fvm_dirichlet_apply(prob.handle, up, float(t), ul, s))
    return u


# --------------------------------------------------------------------------------------
# output side: fluxes across edges and interpolation (src/problem.jl:447-487, src/utils.jl:23-42)
# --------------------------------------------------------------------------------------
def _stored_abg(prob, t, u):
    """alpha, beta, gamma of the stored triangle t (shape_functions.jl:2-19): scalars for a
    vector u, N-tuples for an (N, npoints) u."""
    a, b, c = (int(v) for v in prob.mesh.triangulation.triangles[t])
    s = prob.mesh.props_array[t, :9]
    u = np.asarray(u, dtype=np.float64)
    if u.ndim == 2:
        return tuple(tuple(s[3 * m] * u[l, a] + s[3 * m + 1] * u[l, b] + s[3 * m + 2] * u[l, c] for l in range(u.shape[0]))
                     for m in range(3))
    return tuple(s[3 * m] * u[a] + s[3 * m + 1] * u[b] + s[3 * m + 2] * u[c] for m in range(3))


def construct_flux_function(q, D, Dp):
    """construct_flux_function(q, D, Dp) (src/problem.jl:425-440): q itself when given, else the
    flux of the diffusion function D with parameters Dp,
    (x, y, t, alpha, beta, gamma, p) -> -D(x, y, t, alpha x + beta y + gamma, Dp) (alpha, beta)."""
    if q is not None:
        return q

    def flux(x, y, t, a, b, g, p):
        u = a * x + b * y + g
        d = D(x, y, t, u, Dp)
        return (-d * a, -d * b)

    return flux


def _flux_closures(prob):
    """The flux closure(s) q(x, y, t, alpha, beta, gamma) of a problem (construct_flux_function
    with its parameters bound) or a list of them for a system."""
    if hasattr(prob, "flux_functions"):  # FVMSystem
        return list(prob.flux_functions)
    q = construct_flux_function(prob.flux_function, prob.diffusion_function, prob.diffusion_parameters)
    return ParametrisedFunction(q, prob.flux_parameters)


def compute_flux(prob, i, j, u, t):
    """compute_flux(prob, i, j, u, t) (src/problem.jl:458-487): q . n at the midpoint of edge
    (i, j), n its unit normal rotated clockwise from (i, j) (pointing to the edge's right), q
    the flux of the piecewise-linear u on the triangle to the right of the edge, or on the one
    to its left for a boundary edge with the outside on its right.  For an FVMSystem (u of
    shape (N, npoints)) a tuple of N values, one per component.  Host-side, like the reference."""
    tri = prob.mesh.triangulation
    px, py = tri.points[int(i)]
    qx, qy = tri.points[int(j)]
    ex, ey = qx - px, qy - py
    ell = np.sqrt(ex * ex + ey * ey)
    nx, ny = ey / ell, -ex / ell
    T = tri.edge_triangle(j, i)  # the triangle in the direction of the normal
    if T < 0:
        T = tri.edge_triangle(i, j)
    if T < 0:
        raise ValueError(f"({i}, {j}) is not an edge of the triangulation")
    a, b, g = _stored_abg(prob, T, u)
    mx, my = (px + qx) / 2, (py + qy) / 2
    q = _flux_closures(prob)
    if isinstance(q, list):
        out = []
        for f in q:
            qvx, qvy = f(mx, my, t, a, b, g)
            out.append(nx * qvx + ny * qvy)
        return tuple(out)
    qvx, qvy = q(mx, my, t, a, b, g)
    return nx * qvx + ny * qvy


def _query_points(x, y):
    if y is None:
        xy = x
    else:
        xy = np.stack([np.asarray(x, dtype=np.float64).ravel(), np.asarray(y, dtype=np.float64).ravel()], axis=1)
    if isinstance(xy, np.ndarray):
        return np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
    return xy.reshape(-1, 2).contiguous()


def _like(ref, shape, dtype):
    if isinstance(ref, np.ndarray):
        return np.empty(shape, dtype=dtype)
    import torch

    return torch.empty(shape, dtype=getattr(torch, dtype), device=ref.device)


def interpolate(prob, u, x, y=None, T=None, stream=None):
    """pl_interpolate(prob, T, u, x, y) (src/utils.jl:23-27) for many points at once, on the
    device: each point is located (FVMGeometry.locate, the step the reference's tutorials take
    with jump_and_march) unless the triangles T (caller indices) are given, and u's
    piecewise-linear interpolant is evaluated there; NaN outside the mesh.  `prob` is a problem,
    system, template or FVMGeometry; u (npoints,) or (N, npoints), x, y host arrays (or x an
    (nq, 2) array), or CUDA tensors.  Returns (nq,) or (N, nq) values of u's kind."""
    mesh = prob if isinstance(prob, FVMGeometry) else prob.mesh
    xy = _query_points(x, y)
    nq = xy.shape[0]
    host = isinstance(xy, np.ndarray)
    tri = mesh.locate(xy, stream=stream) if T is None else T
    if host:
        tri = np.ascontiguousarray(tri, dtype=np.int64).reshape(-1)
        uu = np.asarray(u, dtype=np.float64)
        ncomp = 1 if uu.ndim == 1 else uu.shape[0]
        uflat = np.ascontiguousarray(uu.T if uu.ndim == 2 else uu)
    else:
        tri = tri.reshape(-1).to(dtype=getattr(__import__("torch"), "int64")).contiguous()
        ncomp = 1 if u.dim() == 1 else u.shape[0]
        uflat = (u.T if u.dim() == 2 else u).contiguous()
    if tri.shape[0] != nq:
        raise ValueError("T must give one triangle per query point")
    out = _like(xy, (nq, ncomp), "float64")
    up, loc = _lib.array_pointer(uflat)
    tp, _ = _lib.array_pointer(tri, "int64")
    xp, _ = _lib.array_pointer(xy)
    op, _ = _lib.array_pointer(out)
    s = stream if stream is not None else _lib.current_stream_handle()
    check(load().fvm_pl_interpolate(mesh.handle, up, ncomp, nq, tp, xp, op, loc, s))
    return out[:, 0] if ncomp == 1 and (u.ndim if host else u.dim()) == 1 else out.T


def pl_interpolate(prob, T, u, x, y):
    """pl_interpolate(prob, T, u, x, y) (src/utils.jl:23-27): the piecewise-linear interpolant of
    u on triangle T = (i, j, k) (any rotation of a solid triangle) at (x, y); for an (N, npoints)
    u, an array of N values."""
    t = prob.mesh.triangulation.find_triangle(T)
    if t < 0:
        raise ValueError(f"{tuple(T)} is not a solid triangle of the mesh")
    a, b, g = _stored_abg(prob, t, u)
    if isinstance(a, tuple):
        return np.array([a[l] * x + b[l] * y + g[l] for l in range(len(a))])
    return a * x + b * y + g


def two_point_interpolant(mesh, u, i, j, mx, my):
    """two_point_interpolant(mesh, u, i, j, mx, my) (src/utils.jl:36-42): u on the segment from
    node i to node j, linear in the distance from node i."""
    xi, yi = mesh.triangulation.points[int(i)]
    xj, yj = mesh.triangulation.points[int(j)]
    ell = np.sqrt((xj - xi) ** 2 + (yj - yi) ** 2)
    ellp = np.sqrt((mx - xi) ** 2 + (my - yi) ** 2)
    return u[i] + (u[j] - u[i]) * ellp / ell


def jacobian_sparsity(prob, N=None):
    """jacobian_sparsity(prob) (src/solve.jl:50-131): the Jacobian prototype of fvm_eqs!, a
    scipy.sparse CSC matrix of ones.  Node i is coupled to itself and, when it is a vertex, to
    its neighbours in the triangulation.  For an FVMSystem of N equations every coupled node pair
    becomes an N x N block, with unknowns numbered (node - 1) N + component, the reference's
    linear indexing of its N x npoints state.  Takes an FVMProblem, an FVMSystem, a template, or
    a Triangulation (with N for a system) as the reference's methods do."""
    import scipy.sparse as sp

    if isinstance(prob, Triangulation):
        tri = prob
    else:
        tri = prob.mesh.triangulation
        if isinstance(prob, FVMSystem):
            N = prob.neqs
    n = tri.num_points
    T = np.asarray(tri.triangles, dtype=np.int64).reshape(-1, 3)
    diag = np.arange(n, dtype=np.int64)
    rows = np.concatenate([diag, T[:, 0], T[:, 1], T[:, 1], T[:, 2], T[:, 2], T[:, 0]])
    cols = np.concatenate([diag, T[:, 1], T[:, 0], T[:, 2], T[:, 1], T[:, 0], T[:, 2]])
    A = sp.csc_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    A.data[:] = 1.0
    if N is not None:
        A = sp.kron(A, np.ones((int(N), int(N))), format="csc")
    A.sort_indices()
    return A


# --------------------------------------------------------------------------------------
# systems of equations (src/problem.jl:190-365)
# --------------------------------------------------------------------------------------
FLUX_ERROR = """
The flux function errored when evaluated. Please recheck your specification of the function.
If any of your problems have been defined in terms of a diffusion function D(x, y, t, u, p)
rather than a flux function, then you need to instead provide a flux function q(x, y, t, alpha, beta, gamma, p),
recalling the relationship between the two:

    q(x, y, t, alpha, beta, gamma, p) = -D(x, y, t, alpha*x + beta*y + gamma, p) * (alpha, beta)

where p is the same argument for both functions.
"""


class InvalidFluxError(ValueError):
    """A component of an FVMSystem has no usable flux function (src/problem.jl:277-292)."""

    def __init__(self, detail=""):
        super().__init__(FLUX_ERROR + (f"\n{detail}" if detail else ""))


def merge_problem_conditions(probs):
    """merge_problem_conditions (src/problem.jl:336-365): each component keeps its own conditions;
    the condition functions are concatenated component by component, cnum_fncs[i] being the
    number of functions of the components before i; sources and fluxes are wrapped with their
    parameters.  Returns (conditions, cnum_fncs, functions, source_functions, flux_functions)."""
    conditions = tuple(p.conditions for p in probs)
    nf = [len(c.functions) for c in conditions]
    cnum_fncs = tuple(int(v) for v in np.cumsum([0] + nf[:-1]))
    functions = tuple(f for c in conditions for f in c.functions)
    source_functions = tuple(None if p.source_function is None else
                             ParametrisedFunction(p.source_function, p.source_parameters) for p in probs)
    flux_functions = tuple(ParametrisedFunction(p.flux_function, p.flux_parameters) for p in probs)
    return conditions, cnum_fncs, functions, source_functions, flux_functions


class FVMSystem:
    """FVMSystem(prob1, ..., probN) (src/problem.jl:190-365): N coupled equations on one mesh.

    Component i's closures see every component: its flux q(x, y, t, alpha, beta, gamma, p) takes
    N-tuples alpha, beta, gamma (alpha[c] x + beta[c] y + gamma[c] approximates u_c), its source
    and condition functions f(x, y, t, u, p) take u = (u_1, ..., u_N).  Each component keeps its
    own boundary and internal conditions (merge_problem_conditions, :336-365).  Solutions are
    (N, npoints) arrays whose (j, i) entry is component j at node i.

    Device-coded forms (anything else raises UnsupportedFormError at construction):
      flux       -sum_c D_c(x, y) (alpha[c], beta[c])  (diagonal or cross diffusion);
      source     a polynomial of total degree <= 3 in u with (x, y) coefficients;
      Dudt       the same;
      Neumann    affine in u with (x, y) coefficients;
      Dirichlet  a function of (x, y);
    none may depend on t.  A component defined by a diffusion_function raises InvalidFluxError,
    as the reference's construction does."""

    def __init__(self, *probs: FVMProblem):
        if len(probs) == 0:
            raise ValueError("There must be at least one problem.")
        if len(probs) > _lib.FVM_SYSTEM_MAX_EQ:
            raise ValueError(f"at most {_lib.FVM_SYSTEM_MAX_EQ} equations are supported")
        mesh = probs[0].mesh
        if not all(p.mesh is mesh for p in probs):
            raise AssertionError("All problems must have the same mesh.")
        if not all(p.initial_time == probs[0].initial_time for p in probs):
            raise AssertionError("All problems must have the same initial time.")
        if not all(p.final_time == probs[0].final_time for p in probs):
            raise AssertionError("All problems must have the same final time.")
        for i, p in enumerate(probs):
            if p.flux_function is None:
                raise InvalidFluxError(f"component {i} has no flux_function")
        self.mesh = mesh
        self.problems = tuple(probs)
        self.neqs = len(probs)
        self.initial_condition = np.stack([p.initial_condition for p in probs])
        self.initial_time = probs[0].initial_time
        self.final_time = probs[0].final_time
        (self.conditions, self.cnum_fncs, self.functions, self.source_functions,
         self.flux_functions) = merge_problem_conditions(probs)
        self._h = None
        self._build()

    def map_fidx(self, fidx, var):
        """Index into `functions` of component var's condition function fidx (problem.jl:295)."""
        return fidx + self.cnum_fncs[var]

    def _build(self):
        mesh, tri, N = self.mesh, self.mesh.triangulation, self.neqs
        t0 = self.initial_time
        npts, nt, nbe = tri.num_points, tri.num_triangles, tri.num_boundary_edges
        hv = tri.has_vertex()
        dual, quarter = mesh.sample_points()
        dx, dy = dual[..., 0].ravel(), dual[..., 1].ravel()
        qx, qy = quarter[..., 0].ravel(), quarter[..., 1].ravel()
        P = tri.points
        codes = np.zeros((N, npts), dtype=np.int8)
        neu = np.zeros((N, nbe), dtype=np.int8)
        Dd = np.zeros((N, N, 3 * nt))
        Dq = np.zeros((N, N, 2 * nbe))
        basis = monomials(N)
        col = {tuple(e): m for m, e in enumerate(basis)}
        src = np.zeros((N, npts, basis.shape[0]))
        dudt = np.zeros((N, npts, basis.shape[0]))
        qneu = np.zeros((N, 2 * nbe, 1 + N))
        dirv = np.zeros((N, npts))
        tf = self.final_time
        parts = _TimeParts({"time_dirichlet": N * npts, "time_neumann": N * 2 * nbe, "time_source": N * npts,
                            "time_dudt": N * npts})

        def flat(r, sel, size):  # component r's entries of a [N][size] array
            m = np.zeros(N * size, dtype=bool)
            m[r * size:(r + 1) * size] = sel
            return m
        self._codes = codes
        for r, (cond, q) in enumerate(zip(self.conditions, self.flux_functions)):
            code, fidx = cond.vertex_tables(hv)
            nfid = cond.neumann_table(tri.boundary_edges)
            codes[r], neu[r] = code, nfid >= 0
            Dd[r] = classify_system_flux(q, dx, dy, t0, N, f"flux_function of component {r}")
            if nbe:
                Dq[r] = classify_system_flux(q, qx, qy, t0, N, f"flux_function of component {r}")
            free = code == FVM_VERTEX_FREE
            S = self.source_functions[r]
            if S is not None and np.any(free):
                e, c, tp = classify_system_poly(S, P[free, 0], P[free, 1], t0, N, f"source_function of component {r}",
                                                tf=tf, time=True)
                if tp is not None:
                    parts.add("time_source", tp[0], flat(r, free, npts), tp[1])
                for k, ek in enumerate(e):
                    src[r, free, col[tuple(ek)]] = c[:, k]
            for kind, arr, want in (("Dudt", dudt, FVM_VERTEX_DUDT), ("Dirichlet", None, FVM_VERTEX_DIRICHLET)):
                f_of = np.where(code == want, fidx, -1)
                for f in np.unique(f_of[f_of >= 0]):
                    sel = f_of == f
                    what = f"{kind} function {int(f)} of component {r}"
                    e, c, tp = classify_system_poly(cond.functions[int(f)], P[sel, 0], P[sel, 1], t0, N, what,
                                                    max_degree=3 if arr is not None else 0, tf=tf, time=True)
                    if tp is not None:
                        parts.add("time_dudt" if arr is not None else "time_dirichlet", tp[0], flat(r, sel, npts),
                                  tp[1])
                    for k, ek in enumerate(e):
                        if arr is not None:
                            arr[r, sel, col[tuple(ek)]] = c[:, k]
                        else:
                            dirv[r, sel] = c[:, k]
            for f in np.unique(nfid[nfid >= 0]):
                sel = np.repeat(nfid == f, 2)
                e, c, tp = classify_system_poly(cond.functions[int(f)], qx[sel], qy[sel], t0, N,
                                                f"Neumann function {int(f)} of component {r}", max_degree=1, tf=tf,
                                                time=True)
                if tp is not None:
                    parts.add("time_neumann", tp[0], flat(r, sel, 2 * nbe), tp[1])
                for k, ek in enumerate(e):
                    qneu[r, sel, 0 if ek.sum() == 0 else 1 + int(np.argmax(ek))] = c[:, k]
        used = np.nonzero(np.any(src != 0, axis=(0, 1)) | np.any(dudt != 0, axis=(0, 1)))[0]
        self.monomials = basis[used]
        d = _Desc()
        d.c = _lib.SystemDesc()
        d.c.neq = N
        d.arr("vertex_code", as_i8(codes), _lib.c_int8_p)
        d.arr("bedge_neumann", as_i8(neu) if nbe else None, _lib.c_int8_p)
        d.arr("dual_edge_D", as_f64(Dd))
        d.arr("quarter_D", as_f64(Dq) if nbe else None)
        d.c.nmono = int(used.size)
        d.arr("mono_exp", as_i8(basis[used]) if used.size else None, _lib.c_int8_p)
        d.arr("source", as_f64(src[:, :, used]) if used.size and np.any(src) else None)
        d.arr("dudt", as_f64(dudt[:, :, used]) if used.size and np.any(dudt) else None)
        d.arr("quarter_neumann", as_f64(qneu) if nbe and np.any(qneu) else None)
        d.arr("dirichlet", as_f64(dirv) if np.any(dirv) else None)
        parts.fill(d)
        self.time_factors = list(parts.factors)
        h = C.c_void_p()
        check(load().fvm_system_create(mesh.handle, C.byref(d.c), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def info(self) -> Dict[str, int]:
        a = np.zeros(7, dtype=np.int64)
        check(load().fvm_system_info(self._h, dptr(a, _lib.c_int64_p)))
        keys = ["neqs", "flux_blocks", "terms", "varying_terms", "dirichlet_entries", "has_neumann_constants",
                "shared_operator"]
        return dict(zip(keys, (int(v) for v in a)))

    def _flat(self, x, name):
        """(pointer, location, host copy or None) of an (N, npoints) array in the library's
        [point][component] memory order.  numpy arrays of any layout are staged; a CUDA tensor
        must already have that memory order (e.g. torch.empty(npoints, N).T)."""
        N, n = self.neqs, self.mesh.triangulation.num_points
        if tuple(x.shape) != (N, n):
            raise ValueError(f"{name} must have shape ({N}, {n})")
        if isinstance(x, np.ndarray):
            xt = np.ascontiguousarray(x.T, dtype=np.float64)
            return C.c_void_p(xt.ctypes.data), _lib.FVM_PTR_HOST, xt
        p, loc = _lib.array_pointer(x.T)
        return p, loc, None

    def rhs(self, du, u, t=0.0, internal=False, stream=None):
        """fvm_eqs!(du, u, p, t) for the system; u, du (N, npoints).  internal=True takes device
        tensors already in the library's internal point numbering (a device-resident loop's)."""
        up, ul, uh = self._flat(u, "u")  # uh keeps the staged copy alive
        dp, dl, dh = self._flat(du, "du")
        if ul != dl:
            raise TypeError("u and du must both be host arrays or both device tensors")
        if internal:
            if ul != _lib.FVM_PTR_DEVICE:
                raise TypeError("internal=True needs device tensors")
            ul = _lib.FVM_PTR_DEVICE_INTERNAL
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_system_rhs(self._h, up, dp, float(t), ul, s))
        if dh is not None:
            du[...] = dh.T
        return du

    def jvp(self, u, v, t=0.0, stream=None):
        """J(u) v of the system's fvm_eqs! (exact); u, v (N, npoints), returned alike."""
        out = np.empty_like(u) if isinstance(u, np.ndarray) else u.new_empty((u.shape[1], u.shape[0])).T
        up, ul, uh = self._flat(u, "u")  # the staged host copies must outlive the call
        vp, vl, vh = self._flat(v, "v")
        op, ol, oh = self._flat(out, "jv")
        if not (ul == vl == ol):
            raise TypeError("u and v must both be host arrays or both device tensors")
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_system_jvp(self._h, up, vp, op, float(t), ul, s))
        if oh is not None:
            out[...] = oh.T
        return out

    def jacobian_diagonal(self, u, t=0.0, stream=None):
        """diag J(u) of the system's fvm_eqs!, (N, npoints)."""
        out = np.empty_like(u) if isinstance(u, np.ndarray) else u.new_empty((u.shape[1], u.shape[0])).T
        up, ul, uh = self._flat(u, "u")
        op, _, oh = self._flat(out, "diag")
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_system_jacobian_diagonal(self._h, up, op, float(t), ul, s))
        if oh is not None:
            out[...] = oh.T
        return out

    def update_dirichlet_nodes(self, u, t=0.0, stream=None):
        """update_dirichlet_nodes! for the system, in place; u (N, npoints)."""
        up, ul, uh = self._flat(u, "u")
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_system_dirichlet_apply(self._h, up, float(t), ul, s))
        if uh is not None:
            u[...] = uh.T
        return u

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._LIB is not None:
            _lib._LIB.fvm_system_destroy(h)
            self._h = None

    def __repr__(self):
        return f"FVMSystem with {self.neqs} equations and time span ({self.initial_time}, {self.final_time})"


# --------------------------------------------------------------------------------------
# batched instances
# --------------------------------------------------------------------------------------
class BatchedProblem:
    """B instances of a linear FVMProblem that differ only in their diffusion field
    D_b(x, y) (what the reference would run as B FVMProblems, e.g. an EnsembleProblem).

    State arrays are (npoints, B), instance index fastest.  `diffusion_functions` is a
    sequence of closures D_b(x, y, t, u, p) of (x, y) alone, sampled at the dual-edge midpoints
    and boundary quarter points, or an array (B, 3 ntri + 2 nbedge) of those samples.
    precision "fp32" keeps values, state and accumulation in FP32."""

    def __init__(self, prob: FVMProblem, diffusion_functions, diffusion_parameters=None, precision="fp64"):
        mesh = prob.mesh
        tri = mesh.triangulation
        nd, nq = 3 * tri.num_triangles, 2 * tri.num_boundary_edges
        if isinstance(diffusion_functions, np.ndarray):
            Dall = np.ascontiguousarray(diffusion_functions, dtype=np.float64)
            if Dall.ndim != 2 or Dall.shape[1] != nd + nq:
                raise ValueError(f"D samples must be (B, {nd + nq})")
        else:
            dual, quarter = mesh.sample_points()
            pts = np.concatenate([dual.reshape(-1, 2), quarter.reshape(-1, 2)])
            rows = []
            for Db in diffusion_functions:
                c, deg = classify_xytu(ParametrisedFunction(Db, diffusion_parameters), pts[:, 0], pts[:, 1],
                                       prob.initial_time, "batched diffusion_function", max_degree=0)
                rows.append(c[:, 0])
            Dall = np.ascontiguousarray(np.stack(rows))
        self.prob, self.B = prob, Dall.shape[0]
        self.precision = _precision(precision)
        self.dtype = np.float32 if self.precision == FVM_FP32 else np.float64
        dualD = np.ascontiguousarray(Dall[:, :nd])
        quarterD = np.ascontiguousarray(Dall[:, nd:]) if nq else None
        h = C.c_void_p()
        check(load().fvm_batch_create(prob.handle, self.B, dptr(dualD), dptr(quarterD) if quarterD is not None else None,
                                      self.precision, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def rhs(self, du, u, t=0.0, internal=False, stream=None):
        """du[:, b] = fvm_eqs!(u[:, b]) for every instance."""
        dt = "float32" if self.precision == FVM_FP32 else "float64"
        up, ul = _lib.array_pointer(u, dt)
        dp, dl = _lib.array_pointer(du, dt)
        if ul != dl:
            raise TypeError("u and du must both be host arrays or both device tensors")
        if internal:
            if ul != _lib.FVM_PTR_DEVICE:
                raise TypeError("internal=True needs device tensors")
            ul = _lib.FVM_PTR_DEVICE_INTERNAL
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_batch_rhs(self._h, up, dp, float(t), ul, s))
        return du

    def tuning(self):
        a = np.zeros(3, dtype=np.int32)
        check(load().fvm_batch_tuning(self._h, dptr(a, _lib.c_int32_p)))
        return {"block": int(a[0]), "instances_per_thread": int(a[1]), "grid": int(a[2])}

    def solve(self, u0, dt, saveat=None, use_graph=True, stream=None):
        """Fixed-step Tsit5 on every instance; returns (times, array (nsave, npoints, B), stats)."""
        p = self.prob
        ts = _saveat_times(saveat, p.initial_time, p.final_time) if saveat is not None else np.array([p.final_time])
        n = p.mesh.triangulation.num_points
        u0c = np.ascontiguousarray(np.broadcast_to(np.asarray(u0, dtype=np.float64).reshape(n, -1), (n, self.B)))
        out = np.empty((ts.size, n, self.B))
        o = _lib.OdeOptions()
        o.t0, o.tf, o.dt, o.adaptive = p.initial_time, p.final_time, float(dt), 0
        tsc = as_f64(ts)
        o.saveat, o.nsave, o.use_graph = dptr(tsc), ts.size, 1 if use_graph else 0
        st = _lib.OdeStats()
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_batch_tsit5_solve(self._h, dptr(u0c), C.byref(o), dptr(out), C.byref(st), s))
        return ts, out, {"steps": st.naccept, "nrhs": st.nrhs, "elapsed_ms": st.elapsed_ms}

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib._LIB.fvm_batch_destroy(self._h)
            self._h = None


# --------------------------------------------------------------------------------------
# differentiation: discrete adjoint of the time-dependent templates
# --------------------------------------------------------------------------------------
class AdjointProblem:
    """Differentiable batched solve of a DiffusionEquation or LinearReactionDiffusionEquation
    template with respect to a per-vertex log-diffusivity field.

    Instance i has D_i(x, y) = the P1 interpolant of exp(theta[:, i]) over the template's mesh,
    sampled where the reference samples D; conditions, sources and b come from the template (b
    must not depend on D).  Arrays are (npoints, batch) float64, host numpy arrays or CUDA torch
    tensors, in the caller's numbering.  Time stepping is fixed-step Tsit5.  What the reference
    gets by running its solve under ForwardDiff, this gets from a hand-written adjoint:
    `pullback` is the vector-Jacobian product of theta, u0 -> u(T); `loss_and_grad` the same
    for loss = sum (u(T) - u_obs)^2; `rhs_vjp` the one of the right-hand side."""

    def __init__(self, template, batch=1):
        if not isinstance(template, _TimeTemplate):
            raise TypeError("AdjointProblem takes a DiffusionEquation or LinearReactionDiffusionEquation")
        self.template, self.B = template, int(batch)
        self.n = template.mesh.triangulation.num_points
        h = C.c_void_p()
        check(load().fvm_adjoint_create(template.handle, self.B, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def _arrays(self, *xs):
        ptrs, locs = [], set()
        for x in xs:
            if x is None:
                ptrs.append(None)
                continue
            if tuple(x.shape) not in ((self.n, self.B),) and not (self.B == 1 and tuple(x.shape) == (self.n,)):
                raise ValueError(f"arrays must have shape ({self.n}, {self.B})")
            p, loc = _lib.array_pointer(x)
            ptrs.append(p)
            locs.add(loc)
        if len(locs) != 1:
            raise TypeError("arrays must all be host arrays or all CUDA tensors")
        return ptrs, locs.pop()

    def _like(self, x):
        if isinstance(x, np.ndarray):
            return np.empty((self.n, self.B))
        import torch

        return torch.empty((self.n, self.B), dtype=torch.float64, device=x.device)

    @staticmethod
    def _stream(stream):
        return stream if stream is not None else _lib.current_stream_handle()

    def set_log_diffusion(self, theta, stream=None):
        """theta: (npoints, batch) log-diffusivity per vertex and instance."""
        (tp,), loc = self._arrays(theta)
        check(load().fvm_adjoint_set_log_diffusion(self._h, tp, loc, self._stream(stream)))
        return self

    def rhs(self, u, stream=None):
        """A(theta) u + b for every instance."""
        du = self._like(u)
        (up, dp), loc = self._arrays(u, du)
        check(load().fvm_adjoint_rhs(self._h, up, dp, loc, self._stream(stream)))
        return du

    def forward(self, u0, dt, nsteps, stream=None):
        """u(T) after `nsteps` Tsit5 steps of `dt`."""
        uT = self._like(u0)
        (up, tp), loc = self._arrays(u0, uT)
        check(load().fvm_adjoint_forward(self._h, up, float(dt), int(nsteps), tp, loc, self._stream(stream)))
        return uT

    @staticmethod
    def _stats(st):
        return {k: getattr(st, k) for k, _ in _lib.AdjointStats._fields_}

    def pullback(self, u0, dt, nsteps, uT_bar, checkpoint_every=20, stream=None):
        """(theta_bar, u0_bar, stats) = the vector-Jacobian product of u(T) with uT_bar."""
        tb, ub = self._like(u0), self._like(u0)
        (up, bp, tp, ubp), loc = self._arrays(u0, uT_bar, tb, ub)
        st = _lib.AdjointStats()
        check(load().fvm_adjoint_pullback(self._h, up, float(dt), int(nsteps), int(checkpoint_every), bp, tp, ubp,
                                          C.byref(st), loc, self._stream(stream)))
        return tb, ub, self._stats(st)

    def loss_and_grad(self, u0, u_obs, dt, nsteps, checkpoint_every=20, stream=None):
        """(loss (batch,), d loss / d theta, d loss / d u0, stats) for
        loss_i = sum_v (u(T)[v, i] - u_obs[v, i])^2."""
        tb, ub = self._like(u0), self._like(u0)
        (up, op, tp, ubp), loc = self._arrays(u0, u_obs, tb, ub)
        loss = np.empty(self.B)
        st = _lib.AdjointStats()
        check(load().fvm_adjoint_loss_grad(self._h, up, op, float(dt), int(nsteps), int(checkpoint_every),
                                           dptr(loss), tp, ubp, C.byref(st), loc, self._stream(stream)))
        return loss, tb, ub, self._stats(st)

    def rhs_vjp(self, u, w, stream=None):
        """(u_bar, theta_bar) = (A^T w, (d f / d theta)^T w) for f(u, theta) = A(theta) u + b."""
        ub, tb = self._like(u), self._like(u)
        (up, wp, ubp, tp), loc = self._arrays(u, w, ub, tb)
        check(load().fvm_adjoint_rhs_vjp(self._h, up, wp, ubp, tp, loc, self._stream(stream)))
        return ub, tb

    def __del__(self):
        if getattr(self, "_h", None) and _lib._LIB is not None:
            _lib._LIB.fvm_adjoint_destroy(self._h)
            self._h = None


def solve_rrule(adjoint: AdjointProblem, theta, u0, dt, nsteps, checkpoint_every=20):
    """The rrule of theta, u0 -> u(T) in ChainRulesCore's shape: returns (u(T), pullback) where
    pullback(uT_bar) -> (theta_bar, u0_bar)."""
    adjoint.set_log_diffusion(theta)
    uT = adjoint.forward(u0, dt, nsteps)

    def pullback(uT_bar):
        adjoint.set_log_diffusion(theta)
        tb, ub, _ = adjoint.pullback(u0, dt, nsteps, uT_bar, checkpoint_every)
        return tb, ub

    return uT, pullback


# --------------------------------------------------------------------------------------
# templates (src/specific_problems/)
# --------------------------------------------------------------------------------------
class _Template:
    kind = -1
    steady = False

    def _create(self, mesh, BCs, ICs, D, Dp, source=None, source_parameters=None, source_as_reaction=False):
        tri = mesh.triangulation
        self.mesh = mesh
        self.conditions = conds = Conditions(mesh, BCs, ICs)
        hv = tri.has_vertex()
        code, fidx = conds.vertex_tables(hv)
        neu = conds.neumann_table(tri.boundary_edges)
        dual, quarter = mesh.sample_points()
        d = _Desc()
        d.arr("vertex_code", as_i8(code), _lib.c_int8_p)
        d.arr("bedge_neumann", as_i8(neu >= 0), _lib.c_int8_p)
        d.c.diffusion_degree = 0
        d.arr("dual_edge_D", as_f64(sample_xy(D, dual[..., 0].ravel(), dual[..., 1].ravel(), Dp, what="diffusion_function")))
        if tri.num_boundary_edges:
            d.arr("quarter_D", as_f64(sample_xy(D, quarter[..., 0].ravel(), quarter[..., 1].ravel(), Dp,
                                                what="diffusion_function")))
        # condition functions are called with t = u = nothing (abstract_templates.jl:112,131,185)
        fns = conds.functions
        if np.any(neu >= 0):
            qn = np.zeros((tri.num_boundary_edges, 2))
            for f in np.unique(neu[neu >= 0]):
                sel = neu == f
                Q = quarter[sel]
                qn[sel] = sample_xy(fns[int(f)], Q[..., 0].ravel(), Q[..., 1].ravel(), None, None,
                                    what=f"Neumann function {int(f)}").reshape(-1, 2)
            d.c.neumann_degree = 0
            d.arr("quarter_neumann", as_f64(qn.reshape(-1, 1)))
        P = tri.points
        vals = np.zeros(tri.num_points)
        for kind_code in (FVM_VERTEX_DUDT, FVM_VERTEX_DIRICHLET):
            for f in np.unique(fidx[code == kind_code]):
                sel = (code == kind_code) & (fidx == f)
                vals[sel] = sample_xy(fns[int(f)], P[sel, 0], P[sel, 1], None, None, what=f"condition function {int(f)}")
        d.c.dudt_degree = 0
        d.arr("dudt", as_f64(np.where(code == FVM_VERTEX_DUDT, vals, 0.0)))
        self._dirichlet_values = np.where(code == FVM_VERTEX_DIRICHLET, vals, 0.0)
        d.arr("dirichlet", as_f64(self._dirichlet_values))
        if source is not None:
            sv = sample_xy(source, P[:, 0], P[:, 1], source_parameters, what="source_function")
            if source_as_reaction:
                d.c.source_degree = 1
                d.arr("source", as_f64(np.stack([np.zeros_like(sv), sv], axis=1)))
            else:
                d.c.source_degree = 0
                d.arr("source", as_f64(sv))
        d.c.precision = FVM_FP64
        d.c.options = _lib.FVM_PROBLEM_CONDITIONS_ONLY  # the template assembles its own operator
        self._code = code
        hp = C.c_void_p()
        check(load().fvm_problem_create(mesh.handle, C.byref(d.c), C.byref(hp)))
        self._hp = hp
        self._desc = d
        ht = C.c_void_p()
        check(load().fvm_template_create(hp, self.kind, C.byref(ht)))
        self._ht = ht
        self._A = None
        self._b = None

    @property
    def handle(self):
        return self._ht

    def _export(self):
        lib = load()
        nnz = C.c_int64()
        check(lib.fvm_template_export(self._ht, C.byref(nnz), None, None, None, None))
        n = self.mesh.triangulation.num_points
        rowptr = np.empty(n + 1, dtype=np.int32)
        col = np.empty(nnz.value, dtype=np.int32)
        val = np.empty(nnz.value)
        b = np.empty(n)
        check(lib.fvm_template_export(self._ht, C.byref(nnz), dptr(rowptr, _lib.c_int32_p), dptr(col, _lib.c_int32_p),
                                      dptr(val), dptr(b)))
        from scipy.sparse import csr_matrix

        self._A = csr_matrix((val, col, rowptr), shape=(n, n))
        self._b = b

    @property
    def A(self):
        if self._A is None:
            self._export()
        return self._A

    @property
    def b(self):
        if self._b is None:
            self._export()
        return self._b

    def apply(self, du, u, precision="fp64", internal=False, stream=None):
        """du = A u + b: the MatrixOperator product (internal=True: device tensors in the
        library's internal numbering)."""
        up, ul = _lib.array_pointer(u)
        dp, dl = _lib.array_pointer(du)
        if ul != dl:
            raise TypeError("u and du must both be host arrays or both device tensors")
        if internal:
            if ul != _lib.FVM_PTR_DEVICE:
                raise TypeError("internal=True needs device tensors")
            ul = _lib.FVM_PTR_DEVICE_INTERNAL
        s = stream if stream is not None else _lib.current_stream_handle()
        check(load().fvm_template_apply(self._ht, up, dp, _precision(precision), ul, s))
        return du

    def __del__(self):
        if _lib._LIB is None:
            return
        if getattr(self, "_ht", None):
            _lib._LIB.fvm_template_destroy(self._ht)
            self._ht = None
        if getattr(self, "_hp", None):
            _lib._LIB.fvm_problem_destroy(self._hp)
            self._hp = None


class _TimeTemplate(_Template):
    def _init_time(self, initial_condition, initial_time, final_time):
        ic = np.array(initial_condition, dtype=np.float64)
        if ic.shape[0] != self.mesh.triangulation.num_points:
            raise AssertionError("initial condition length must equal the number of points")
        self.initial_condition = ic
        # apply_dirichlet_conditions! (abstract_templates.jl:109-117)
        u0 = ic.copy()
        dmask = self._code == FVM_VERTEX_DIRICHLET
        u0[dmask] = self._dirichlet_values[dmask]
        self.u0 = u0
        self.initial_time = float(initial_time)
        self.final_time = float(final_time)


class DiffusionEquation(_TimeTemplate):
    """DiffusionEquation (src/specific_problems/diffusion_equation.jl:49-101):
    du/dt = A u + b.  Solutions carry the reference's extra last component (= 1)."""

    kind = _lib.FVM_TEMPLATE_DIFFUSION

    def __init__(self, mesh, BCs, ICs=None, *, diffusion_function, diffusion_parameters=None, initial_condition,
                 initial_time=0.0, final_time, **kwargs):
        self.diffusion_function, self.diffusion_parameters = diffusion_function, diffusion_parameters
        self._create(mesh, BCs, ICs, diffusion_function, diffusion_parameters)
        self._init_time(initial_condition, initial_time, final_time)

    def __repr__(self):
        return f"DiffusionEquation with {self.mesh.triangulation.num_points} nodes and time span ({self.initial_time}, {self.final_time})"


class LinearReactionDiffusionEquation(_TimeTemplate):
    """LinearReactionDiffusionEquation (linear_reaction_diffusion_equations.jl:53-125):
    du/dt = div(D grad u) + f(x) u."""

    kind = _lib.FVM_TEMPLATE_LINEAR_REACTION_DIFFUSION

    def __init__(self, mesh, BCs, ICs=None, *, diffusion_function, diffusion_parameters=None, source_function,
                 source_parameters=None, initial_condition, initial_time=0.0, final_time, **kwargs):
        self.diffusion_function, self.diffusion_parameters = diffusion_function, diffusion_parameters
        self.source_function, self.source_parameters = source_function, source_parameters
        self._create(mesh, BCs, ICs, diffusion_function, diffusion_parameters, source_function, source_parameters,
                     source_as_reaction=True)
        self._init_time(initial_condition, initial_time, final_time)


class PoissonsEquation(_Template):
    """PoissonsEquation (poissons_equation.jl:42-88): div(D grad u) = f, A u = b."""

    kind = _lib.FVM_TEMPLATE_POISSON
    steady = True

    def __init__(self, mesh, BCs, ICs=None, *, diffusion_function=lambda x, y, p: 1.0 + 0.0 * x,
                 diffusion_parameters=None, source_function, source_parameters=None, **kwargs):
        self.diffusion_function, self.diffusion_parameters = diffusion_function, diffusion_parameters
        self.source_function, self.source_parameters = source_function, source_parameters
        self._create(mesh, BCs, ICs, diffusion_function, diffusion_parameters, source_function, source_parameters)


class LaplacesEquation(PoissonsEquation):
    """LaplacesEquation (laplaces_equation.jl:48-94): div(D grad u) = 0, assembled as the Poisson
    template's A with b holding only the boundary terms (the Poisson template with f = 0)."""

    def __init__(self, mesh, BCs, ICs=None, *, diffusion_function=lambda x, y, p: 1.0 + 0.0 * x,
                 diffusion_parameters=None, **kwargs):
        super().__init__(mesh, BCs, ICs, diffusion_function=diffusion_function,
                         diffusion_parameters=diffusion_parameters, source_function=lambda x, y, p: 0.0 * x)


class MeanExitTimeProblem(_Template):
    """MeanExitTimeProblem (mean_exit_time.jl:43-94): div(D grad T) = -1."""

    kind = _lib.FVM_TEMPLATE_MEAN_EXIT_TIME
    steady = True

    def __init__(self, mesh, BCs, ICs=None, *, diffusion_function, diffusion_parameters=None, **kwargs):
        conds = Conditions(mesh, BCs, ICs)
        if conds.has_dudt_nodes():
            raise ValueError("MeanExitTimeProblem does not support Dudt nodes.")
        if conds.has_constrained_edges():
            raise ValueError("MeanExitTimeProblem does not support Constrained edges.")
        self.diffusion_function, self.diffusion_parameters = diffusion_function, diffusion_parameters
        self._create(mesh, BCs, ICs, diffusion_function, diffusion_parameters)


# --------------------------------------------------------------------------------------
# solve
# --------------------------------------------------------------------------------------
class Tsit5:
    """Tsitouras 5(4) explicit Runge-Kutta (the algorithm the reference's README uses)."""

    def __repr__(self):
        return "Tsit5()"


class TRBDF2:
    """TR-BDF2 (the implicit method of the reference's tutorials), on the device: simplified
    Newton per stage, matrix-free BiCGStab on W = I - d h J with the exact Jacobian-vector
    product of fvm_eqs!, diag(W) as preconditioner; adaptive with TR-BDF2's error estimate
    (dt given with adaptive=False: fixed steps).  FVMProblem, FVMSystem, DiffusionEquation and
    LinearReactionDiffusionEquation (J = A)."""

    def __repr__(self):
        return "TRBDF2()"


class SteadyFVMProblem:
    """SteadyFVMProblem(prob) (src/problem.jl:166-180): an FVMProblem or FVMSystem to be solved for
    du/dt = 0.  The problem's initial condition is the initial guess, and its final time is
    conventionally Inf.  solve(steady, DynamicSS(...)) or solve(steady, NewtonRaphson())."""

    def __init__(self, prob):
        if not isinstance(prob, (FVMProblem, FVMSystem)):
            raise TypeError("SteadyFVMProblem wraps an FVMProblem or an FVMSystem")
        self.problem = prob
        self.mesh = prob.mesh

    def __repr__(self):
        nv = int(self.mesh.triangulation.has_vertex().sum())
        if isinstance(self.problem, FVMSystem):
            return f"SteadyFVMProblem with {nv} nodes and {self.problem.neqs} equations"
        return f"SteadyFVMProblem with {nv} nodes"


@dataclass
class DynamicSS:
    """DynamicSS(alg; abstol = 1e-8, reltol = 1e-6, tspan = Inf) of SteadyStateDiffEq: step the
    ODE in pseudo-time from the initial guess, the Dirichlet update after every step, until
    max|du/dt| <= abstol or max|du/dt| <= reltol max|du/dt + u|.  The device integrator is
    TR-BDF2 whichever implicit method `alg` names (the tutorials use TRBDF2 and Rosenbrock23):
    the steady state is the same, the path to it differs.  ode_abstol / ode_reltol are the
    integrator's step tolerances."""

    alg: Any = None
    abstol: float = 1e-8
    reltol: float = 1e-6
    tspan: float = float("inf")
    ode_abstol: float = 1e-6
    ode_reltol: float = 1e-3
    max_steps: int = 0


@dataclass
class NewtonRaphson:
    """NewtonRaphson() of NonlinearSolve on f(u) = 0, on the device: each iteration solves
    (F - J(u)) du = f(u) by matrix-free BiCGStab with the exact JVP, F the identity on the rows
    the problem fixes (Dirichlet nodes, points outside the mesh), which keep their values (the
    Dirichlet values at the initial time are applied to the guess first).  Stops when
    max|f(u)| <= abstol or <= reltol max|f(u) + u|."""

    abstol: float = 1e-10
    reltol: float = 1e-10
    max_iters: int = 50


@dataclass
class SteadyStateSolution:
    """The steady state: u (vector, or N x npoints matrix for a system), stats, retcode."""

    u: np.ndarray
    stats: Dict[str, Any] = field(default_factory=dict)
    retcode: str = "Success"


def _solve_steady(sp, alg, abstol, reltol, stream):
    """solve(::SteadyFVMProblem, alg) (src/solve.jl:184-196) on the device."""
    prob = sp.problem
    alg = alg if alg is not None else DynamicSS(TRBDF2())
    o = _lib.SteadyOptions()
    if isinstance(alg, NewtonRaphson):
        o.method = _lib.FVM_STEADY_NEWTON
        o.max_iters = int(alg.max_iters)
        method = "newton"
    elif isinstance(alg, DynamicSS):
        o.method = _lib.FVM_STEADY_DYNAMIC
        o.tmax = prob.initial_time + float(alg.tspan)
        o.ode_abstol, o.ode_reltol = alg.ode_abstol, alg.ode_reltol
        o.max_iters = int(alg.max_steps)
        method = "dynamic"
    else:
        raise TypeError("a SteadyFVMProblem is solved with DynamicSS(...) or NewtonRaphson()")
    o.abstol = float(alg.abstol if abstol is None else abstol)
    o.reltol = float(alg.reltol if reltol is None else reltol)
    o.t = prob.initial_time
    st = _lib.SteadyStats()
    lib = load()
    if isinstance(prob, FVMSystem):
        u0 = as_f64(prob.initial_condition.T)  # [point][component]
        out = _lib.host_empty(u0.shape)
        status = lib.fvm_system_steady_solve(prob.handle, dptr(u0), C.byref(o), dptr(out), C.byref(st), stream)
        u = out.T
    else:
        u0 = as_f64(prob.initial_condition)
        out = _lib.host_empty(u0.shape)
        status = lib.fvm_steady_solve(prob.handle, dptr(u0), C.byref(o), dptr(out), C.byref(st), stream)
        u = out
    stats = {"method": method, "iterations": st.iterations, "krylov_iters": st.krylov_iters, "jvps": st.jvps,
             "nrhs": st.nrhs, "residual": st.residual, "t_final": st.t_final, "elapsed_ms": st.elapsed_ms}
    sol = SteadyStateSolution(u, stats)
    try:
        check(status)
    except _lib.NotConvergedError as e:
        sol.retcode = "Failure"
        e.solution = sol  # the last iterate and its statistics
        raise
    return sol


def jvp(prob, u, v, t=0.0, stream=None):
    """J(u) v, the Jacobian-vector product of fvm_eqs! (exact for every device-coded form).
    u, v host float64 arrays or CUDA tensors (caller numbering); returns J(u) v of their kind."""
    prob = _prob_of(prob)
    if isinstance(prob, FVMSystem):
        return prob.jvp(u, v, t, stream)
    out = np.empty_like(u) if isinstance(u, np.ndarray) else u.new_empty(u.shape)
    up, ul = _lib.array_pointer(u)
    vp, vl = _lib.array_pointer(v)
    op, ol = _lib.array_pointer(out)
    if not (ul == vl == ol):
        raise TypeError("u and v must both be host arrays or both device tensors")
    s = stream if stream is not None else _lib.current_stream_handle()
    check(load().fvm_jvp(prob.handle, up, vp, op, float(t), ul, s))
    return out


def jacobian_diagonal(prob, u, t=0.0, stream=None):
    """diag J(u) of fvm_eqs! (the Jacobi preconditioner of a Newton-Krylov solve)."""
    prob = _prob_of(prob)
    if isinstance(prob, FVMSystem):
        return prob.jacobian_diagonal(u, t, stream)
    out = np.empty_like(u) if isinstance(u, np.ndarray) else u.new_empty(u.shape)
    up, ul = _lib.array_pointer(u)
    op, _ = _lib.array_pointer(out)
    s = stream if stream is not None else _lib.current_stream_handle()
    check(load().fvm_jacobian_diagonal(prob.handle, up, op, float(t), ul, s))
    return out


@dataclass
class KrylovSolver:
    """GPU steady solver: method "auto" (CG if symmetric, else BiCGStab), "cg", "bicgstab";
    precond "jacobi" or "chebyshev" (a degree-`cheb_degree` Chebyshev polynomial in the
    Jacobi-scaled operator); mode "fp64", "mixed" or "fp32_precond".  "mixed" with the
    Chebyshev preconditioner runs the Krylov iteration in FP64 and evaluates the polynomial in
    FP32 (values, vectors, difference-form products); with Jacobi it runs FP32 Krylov cycles,
    each reducing the residual by `inner_reduction`, folded into the FP64 solution.
    "fp32_precond": FP64 iteration and arithmetic, the polynomial reading FP32-stored values.
    The stopping test is ||b - A x|| / ||b|| <= rtol for the FP64 solution, evaluated in FP64
    in difference form with compensated row sums."""

    mode: str = "fp64"
    method: str = "auto"
    rtol: float = 1e-10
    max_iters: int = 1_000_000
    inner_reduction: float = 1e-3
    precond: str = "jacobi"
    cheb_degree: int = 4


@dataclass
class ODESolution:
    t: np.ndarray
    u: list
    stats: Dict[str, Any] = field(default_factory=dict)
    retcode: str = "Success"

    def __getitem__(self, i):
        return self.u[i]

    def __len__(self):
        return len(self.u)


@dataclass
class LinearSolution:
    u: np.ndarray
    stats: Dict[str, Any] = field(default_factory=dict)
    retcode: str = "Success"


_DRIVERS = {0: "host", 1: "fixed_graph", 2: "device_loop", 3: "cluster"}


def _saveat_times(saveat, t0, tf):
    if saveat is None:
        return np.array([t0, tf])
    if np.isscalar(saveat):
        step = float(saveat)
        n = int(np.floor((tf - t0) / step + 1e-9))
        ts = t0 + step * np.arange(n + 1)
        if ts[-1] < tf - 1e-12 * max(1.0, abs(tf)):
            ts = np.append(ts, tf)
        return ts
    return np.asarray(saveat, dtype=np.float64)


def solve(prob, alg=None, *, saveat=None, dt=None, adaptive=None, abstol=None, reltol=None, max_steps=0,
          use_graph=True, parallel=True, precision="fp64", stream=None, **kwargs):
    """solve(prob, alg; saveat, ...) (src/solve.jl:184-220; abstract_templates.jl:58-60).

    Time-dependent problems step with Tsit5 or TRBDF2 (adaptive unless `dt` is given with
    adaptive=False; abstol 1e-6, reltol 1e-3 by default); steady templates solve A u = b with the
    GPU Krylov solver; a SteadyFVMProblem takes DynamicSS or NewtonRaphson (abstol / reltol
    then override the method's own)."""
    lib = load()
    s = stream if stream is not None else _lib.current_stream_handle()
    if isinstance(prob, SteadyFVMProblem):
        return _solve_steady(prob, alg, abstol, reltol, s)
    abstol = 1e-6 if abstol is None else abstol
    reltol = 1e-3 if reltol is None else reltol
    if isinstance(prob, (FVMProblem, FVMSystem)) and not np.isfinite(prob.final_time):
        raise ValueError("the final time is not finite: wrap the problem in SteadyFVMProblem for its steady state")
    if isinstance(prob, _Template) and prob.steady:
        opt = alg if isinstance(alg, KrylovSolver) else KrylovSolver()
        so = _lib.SolverOptions()
        so.rtol = opt.rtol
        so.max_iters = opt.max_iters
        so.method = {"auto": _lib.FVM_SOLVER_AUTO, "cg": _lib.FVM_SOLVER_CG,
                     "bicgstab": _lib.FVM_SOLVER_BICGSTAB}[opt.method]
        so.precond = {"jacobi": _lib.FVM_PRECOND_JACOBI, "chebyshev": _lib.FVM_PRECOND_CHEBYSHEV}[opt.precond]
        so.cheb_degree = int(opt.cheb_degree)
        so.mode = {"fp64": _lib.FVM_SOLVE_FP64, "mixed": _lib.FVM_SOLVE_MIXED,
                   "fp32_precond": _lib.FVM_SOLVE_FP32_PRECOND}[opt.mode]
        so.inner_reduction = opt.inner_reduction
        x = np.zeros(prob.mesh.triangulation.num_points)
        st = _lib.SolverStats()
        status = lib.fvm_template_steady_solve(prob.handle, C.c_void_p(x.ctypes.data), C.byref(so), C.byref(st),
                                               _lib.FVM_PTR_HOST, s)
        sol = LinearSolution(x, {"iterations": st.iterations, "refinements": st.refinements,
                                 "rel_residual": st.rel_residual, "elapsed_ms": st.elapsed_ms,
                                 "method": "cg" if st.method_used == _lib.FVM_SOLVER_CG else "bicgstab",
                                 "symmetric": bool(st.symmetric), "fallback_fp64": bool(st.fallback_fp64)})
        try:
            check(status)
        except _lib.NotConvergedError as e:
            e.solution = sol  # the last iterate and its statistics
            raise
        return sol
    if isinstance(prob, _TimeTemplate):
        t0, tf, u0 = prob.initial_time, prob.final_time, prob.u0
    elif isinstance(prob, FVMProblem):
        t0, tf, u0 = prob.initial_time, prob.final_time, prob.initial_condition
    elif isinstance(prob, FVMSystem):
        t0, tf, u0 = prob.initial_time, prob.final_time, prob.initial_condition.T  # [point][component]
    else:
        raise TypeError(f"cannot solve {type(prob).__name__}")
    ts = _saveat_times(saveat, t0, tf)
    n = prob.mesh.triangulation.num_points
    out = _lib.host_empty((ts.size, n, prob.neqs) if isinstance(prob, FVMSystem) else (ts.size, n))
    o = _lib.OdeOptions()
    o.t0, o.tf = t0, tf
    if adaptive is None:
        adaptive = dt is None
    o.adaptive = 1 if adaptive else 0
    o.dt = float(dt) if dt is not None else 0.0
    o.abstol, o.reltol = abstol, reltol
    o.max_steps = int(max_steps)
    tsc = as_f64(ts)
    o.saveat = dptr(tsc)
    o.nsave = ts.size
    o.use_graph = 1 if use_graph else 0
    o.precision = _precision(precision)
    st = _lib.OdeStats()
    u0c = as_f64(u0)
    if isinstance(prob, _TimeTemplate) and isinstance(alg, TRBDF2):
        ist = _lib.ImplicitStats()
        check(lib.fvm_template_trbdf2_solve(prob.handle, dptr(u0c), C.byref(o), dptr(out), C.byref(st), C.byref(ist),
                                            s))
        us = [np.append(row, 1.0) for row in out]
        return ODESolution(ts, us, {"naccept": st.naccept, "nreject": st.nreject, "nrhs": st.nrhs,
                                    "t_final": st.t_final, "elapsed_ms": st.elapsed_ms, "driver": "host",
                                    "newton_iters": ist.newton_iters, "krylov_iters": ist.krylov_iters,
                                    "jvps": ist.jvps, "newton_failures": ist.newton_failures})
    if isinstance(prob, _TimeTemplate):
        check(lib.fvm_template_tsit5_solve(prob.handle, dptr(u0c), C.byref(o), dptr(out), C.byref(st), s))
        us = [np.append(row, 1.0) for row in out]  # the augmented component of the MatrixOperator form
    elif isinstance(prob, FVMSystem) and isinstance(alg, TRBDF2):
        ist = _lib.ImplicitStats()
        check(lib.fvm_system_trbdf2_solve(prob.handle, dptr(u0c), C.byref(o), dptr(out), C.byref(st), C.byref(ist),
                                          s))
        return ODESolution(ts, [row.T for row in out],
                           {"naccept": st.naccept, "nreject": st.nreject, "nrhs": st.nrhs, "t_final": st.t_final,
                            "elapsed_ms": st.elapsed_ms, "driver": "host", "newton_iters": ist.newton_iters,
                            "krylov_iters": ist.krylov_iters, "jvps": ist.jvps,
                            "newton_failures": ist.newton_failures})
    elif isinstance(prob, FVMSystem):
        check(lib.fvm_system_tsit5_solve(prob.handle, dptr(u0c), C.byref(o), dptr(out), C.byref(st), s))
        us = [row.T for row in out]  # (N, npoints) views: entry (j, i) is component j at node i
    elif isinstance(alg, TRBDF2):
        if not isinstance(prob, FVMProblem):
            raise TypeError("TRBDF2 runs on an FVMProblem, an FVMSystem or a time-dependent template")
        ist = _lib.ImplicitStats()
        check(lib.fvm_trbdf2_solve(prob.handle, dptr(u0c), C.byref(o), dptr(out), C.byref(st), C.byref(ist), s))
        us = list(out)
        return ODESolution(ts, us, {"naccept": st.naccept, "nreject": st.nreject, "nrhs": st.nrhs,
                                    "t_final": st.t_final, "elapsed_ms": st.elapsed_ms, "driver": "host",
                                    "newton_iters": ist.newton_iters, "krylov_iters": ist.krylov_iters,
                                    "jvps": ist.jvps, "newton_failures": ist.newton_failures})
    else:
        check(lib.fvm_tsit5_solve(prob.handle, dptr(u0c), C.byref(o), dptr(out), C.byref(st), s))
        us = list(out)  # rows of the one output array, not copies
    return ODESolution(ts, us, {"naccept": st.naccept, "nreject": st.nreject, "nrhs": st.nrhs,
                                "t_final": st.t_final, "elapsed_ms": st.elapsed_ms,
                                "driver": _DRIVERS.get(st.driver, str(st.driver))})
