"""Triangulations for the finite-volume path.

The reference takes its meshes from DelaunayTriangulation.jl (>= 1.6.6, not
vendored).  This module restates the small part of that package the hot path
needs: a `Triangulation` holding points, solid triangles (counter-clockwise)
and boundary segments, plus the generators used by the reference's tests and
documentation.

Numbering facts pinned by the reference's own tests:

* `triangulate_rectangle(a, b, c, d, nx, ny)` numbers vertex (i, j) (1-based)
  as `i + (j - 1) * nx`, x fastest (test/test_functions.jl:112 builds internal
  Dirichlet nodes as `7 + (i - 1) * 12` on a 12 x 19 mesh).
* each lattice cell is split along its (i+1, j)-(i, j+1) diagonal: the
  200 x 200 corner test uses triangle `(1, 2, 201)` (test/equations.jl:42).
* with `single_boundary=false` the four segments are bottom, right, top, left
  (test/test_functions.jl:590-597 maps them to boundary indices 1..4).

All indices here are 0-based (Python); the C ABI is 0-based too.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "Triangulation",
    "triangulate_rectangle",
    "triangulate_annulus",
    "triangulate_disk",
    "triangulate_points",
]


class Triangulation:
    """Points, solid triangles and boundary segments of a 2D mesh.

    Stands in for DelaunayTriangulation.jl's `Triangulation` on the hot path:
    `each_solid_triangle`, `get_boundary_edge_map`, `get_adjacent(tri, i, j)`
    for boundary edges, `has_vertex`, `num_ghost_vertices`.

    Parameters
    ----------
    points : (npoints, 2) float64
    triangles : (ntri, 3) int, counter-clockwise, 0-based
    boundary_nodes : list of segments; each segment is a sequence of vertex
        indices walked with the domain on the left.  Segment ``s`` has ghost
        vertex ``-(s + 1)`` in the reference's numbering and owns the boundary
        condition with (1-based) index ``s + 1``.
    """

    def __init__(self, points, triangles, boundary_nodes):
        self.points = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 2))
        tris = np.ascontiguousarray(np.asarray(triangles, dtype=np.int64).reshape(-1, 3))
        self.triangles = tris
        self.boundary_nodes = [np.asarray(s, dtype=np.int64) for s in boundary_nodes]
        self._build_boundary()

    # -- reference-like queries -------------------------------------------------
    @property
    def num_points(self) -> int:
        return self.points.shape[0]

    @property
    def num_triangles(self) -> int:
        return self.triangles.shape[0]

    @property
    def num_boundary_edges(self) -> int:
        return self.boundary_edges.shape[0]

    @property
    def num_ghost_vertices(self) -> int:
        """Number of boundary segments (DelaunayTriangulation.num_ghost_vertices)."""
        return len(self.boundary_nodes)

    def has_vertex(self) -> np.ndarray:
        """Boolean mask: point i is a vertex of some solid triangle."""
        m = np.zeros(self.num_points, dtype=bool)
        m[self.triangles.ravel()] = True
        return m

    def edge_triangle(self, i, j) -> int:
        """Index of the solid triangle holding the oriented edge (i, j) (its third vertex is
        get_adjacent(tri, i, j)), or -1 when (i, j) has the outside on its left."""
        if not hasattr(self, "_edge_keys"):
            t = self.triangles
            n = max(self.num_points, 1)
            keys = np.concatenate([t[:, 0] * n + t[:, 1], t[:, 1] * n + t[:, 2], t[:, 2] * n + t[:, 0]])
            order = np.argsort(keys, kind="stable")
            self._edge_keys = keys[order]
            self._edge_tri = order % max(self.num_triangles, 1)
        n = max(self.num_points, 1)
        q = int(i) * n + int(j)
        pos = int(np.searchsorted(self._edge_keys, q))
        if pos < self._edge_keys.size and self._edge_keys[pos] == q:
            return int(self._edge_tri[pos])
        return -1

    def find_triangle(self, T) -> int:
        """Index of the stored solid triangle that is (i, j, k) up to rotation, or -1."""
        i, j, k = (int(v) for v in T)
        t = self.edge_triangle(i, j)
        return t if t >= 0 and k in self.triangles[t] else -1

    # -- boundary edge map ------------------------------------------------------
    def _build_boundary(self):
        edges, seg = [], []
        for s, nodes in enumerate(self.boundary_nodes):
            for a in range(len(nodes) - 1):
                edges.append((nodes[a], nodes[a + 1]))
                seg.append(s)
        self.boundary_edges = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
        self.boundary_segment = np.asarray(seg, dtype=np.int64)
        # get_adjacent(tri, i, j): the third vertex k of the solid triangle
        # containing the oriented edge (i, j)
        t = self.triangles
        n = max(self.num_points, 1)
        keys = np.concatenate([t[:, 0] * n + t[:, 1], t[:, 1] * n + t[:, 2], t[:, 2] * n + t[:, 0]])
        third = np.concatenate([t[:, 2], t[:, 0], t[:, 1]])
        order = np.argsort(keys, kind="stable")
        skeys = keys[order]
        q = self.boundary_edges[:, 0] * n + self.boundary_edges[:, 1]
        pos = np.searchsorted(skeys, q)
        ok = (pos < skeys.size) & (skeys[np.minimum(pos, skeys.size - 1)] == q) if skeys.size else np.zeros(q.size, bool)
        if not np.all(ok):
            bad = self.boundary_edges[~ok][:3]
            raise ValueError(f"boundary edges {bad.tolist()} are not oriented with a solid triangle on their left")
        self.boundary_adjacent = third[order[pos]] if q.size else np.zeros(0, dtype=np.int64)


def disjoint_union(tris):
    """One Triangulation holding several meshes side by side (no shared points).

    Mesh m's points are offset by the point counts of the meshes before it; its boundary
    segments follow those of the meshes before it.  A problem on the union is block-diagonal,
    so one launch per RHS (one captured graph per Tsit5 step) advances every mesh: the
    multi-mesh batch of uneven sizes.  Returns (union, point offsets, segment offsets)."""
    pts, trs, segs = [], [], []
    poff, soff = [0], [0]
    for t in tris:
        o = poff[-1]
        pts.append(t.points)
        trs.append(t.triangles + o)
        segs += [np.asarray(s) + o for s in t.boundary_nodes]
        poff.append(o + t.num_points)
        soff.append(soff[-1] + t.num_ghost_vertices)
    return Triangulation(np.concatenate(pts), np.concatenate(trs), segs), np.array(poff), np.array(soff)


def _orient_ccw(points, tris):
    p, q, r = points[tris[:, 0]], points[tris[:, 1]], points[tris[:, 2]]
    det = (q[:, 0] - p[:, 0]) * (r[:, 1] - p[:, 1]) - (q[:, 1] - p[:, 1]) * (r[:, 0] - p[:, 0])
    tris = tris.copy()
    cw = det < 0
    tris[cw, 1], tris[cw, 2] = tris[cw, 2].copy(), tris[cw, 1].copy()
    return tris


def triangulate_rectangle(a, b, c, d, nx, ny, single_boundary=False):
    """Lattice triangulation of [a, b] x [c, d] with nx * ny points.

    Restates DelaunayTriangulation.jl's `triangulate_rectangle`: points
    `(a + (i-1)dx, c + (j-1)dy)` with index `i + (j-1)nx` (x fastest),
    two triangles per cell, `(i,j),(i+1,j),(i,j+1)` and
    `(i+1,j),(i+1,j+1),(i,j+1)`; boundary walked counter-clockwise from the
    bottom-left corner, as one segment or as four (bottom, right, top, left).
    Coordinates may differ from DelaunayTriangulation.jl's in the last ulp.
    """
    nx, ny = int(nx), int(ny)
    if nx < 2 or ny < 2:
        raise ValueError("triangulate_rectangle needs nx >= 2 and ny >= 2")
    dx = (b - a) / (nx - 1)
    dy = (d - c) / (ny - 1)
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny))  # (ny, nx)
    pts = np.empty((nx * ny, 2))
    pts[:, 0] = (a + ii * dx).ravel()
    pts[:, 1] = (c + jj * dy).ravel()
    pts[(ii == nx - 1).ravel(), 0] = b
    pts[(jj == ny - 1).ravel(), 1] = d
    ci, cj = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1))
    ci, cj = ci.ravel(), cj.ravel()
    v00 = ci + cj * nx
    v10 = v00 + 1
    v01 = v00 + nx
    v11 = v01 + 1
    t1 = np.stack([v00, v10, v01], axis=1)
    t2 = np.stack([v10, v11, v01], axis=1)
    tris = np.empty((2 * t1.shape[0], 3), dtype=np.int64)
    tris[0::2] = t1
    tris[1::2] = t2
    bottom = np.arange(nx)
    right = (nx - 1) + nx * np.arange(ny)
    top = (nx * (ny - 1)) + np.arange(nx - 1, -1, -1)
    left = nx * np.arange(ny - 1, -1, -1)
    if single_boundary:
        seg = np.concatenate([bottom, right[1:], top[1:], left[1:]])
        segments = [seg]
    else:
        segments = [bottom, right, top, left]
    return Triangulation(pts, tris, segments)


def triangulate_annulus(r_inner, r_outer, nr, ntheta, nsegments=4):
    """Structured annulus mesh (polar lattice split into triangles).

    Stand-in for the reference's test annulus (test/test_functions.jl:52-67,
    a constrained Delaunay triangulation of radii 1 and 1/2 with each circle in
    4 quarter segments).  Outer circle walked counter-clockwise, inner circle
    clockwise; each circle split into `nsegments` segments of equal angle, outer
    segments first.
    """
    nr, ntheta = int(nr), int(ntheta)
    if ntheta % nsegments:
        raise ValueError("ntheta must be a multiple of nsegments")
    th = 2 * np.pi * np.arange(ntheta) / ntheta
    r = np.linspace(r_inner, r_outer, nr)
    R, TH = np.meshgrid(r, th, indexing="ij")  # (nr, ntheta)
    pts = np.stack([(R * np.cos(TH)).ravel(), (R * np.sin(TH)).ravel()], axis=1)
    idx = lambda a, k: a * ntheta + (k % ntheta)  # noqa: E731
    tris = []
    for a in range(nr - 1):
        for k in range(ntheta):
            p00, p01 = idx(a, k), idx(a, k + 1)
            p10, p11 = idx(a + 1, k), idx(a + 1, k + 1)
            tris.append((p00, p01, p10))
            tris.append((p01, p11, p10))
    tris = _orient_ccw(pts, np.asarray(tris, dtype=np.int64))
    per = ntheta // nsegments
    outer = [idx(nr - 1, k) for k in range(ntheta + 1)]
    inner = [idx(0, ntheta - k) for k in range(ntheta + 1)]
    segs = [outer[s * per:(s + 1) * per + 1] for s in range(nsegments)]
    segs += [inner[s * per:(s + 1) * per + 1] for s in range(nsegments)]
    return Triangulation(pts, tris, segs)


def triangulate_points(points, boundary_nodes=None):
    """Delaunay triangulation (scipy Qhull) of a convex point set.

    Triangles are re-oriented counter-clockwise.  Without `boundary_nodes` the
    convex hull, walked counter-clockwise, is the single boundary segment.
    """
    from scipy.spatial import Delaunay

    pts = np.asarray(points, dtype=np.float64)
    dl = Delaunay(pts)
    tris = _orient_ccw(pts, dl.simplices.astype(np.int64))
    if boundary_nodes is None:
        hull = dl.convex_hull  # (h, 2) unordered
        nxt = {}
        # orient each hull edge so that the owning triangle lies on its left
        tri_of = {}
        for t in tris:
            for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
                tri_of[(a, b)] = True
        for a, b in hull:
            if (a, b) in tri_of:
                nxt[a] = b
            else:
                nxt[b] = a
        start = min(nxt)
        seg = [start]
        v = nxt[start]
        while v != start:
            seg.append(v)
            v = nxt[v]
        seg.append(start)
        boundary_nodes = [seg]
    return Triangulation(pts, tris, boundary_nodes)


def triangulate_disk(n_interior, n_boundary, seed=0, radius=1.0):
    """Delaunay mesh of `n_interior` uniform random points in a disk plus
    `n_boundary` equispaced boundary points (one boundary segment).

    Interior points use r = R sqrt(U) with R = radius * cos(pi / n_boundary)
    * (1 - 1e-9), so every point lies inside the inscribed polygon and the
    convex hull is exactly the boundary polygon.  Point order: boundary points
    first (counter-clockwise from angle 0), then interior points.
    """
    rng = np.random.default_rng(seed)
    nb = int(n_boundary)
    th = 2 * np.pi * np.arange(nb) / nb
    bpts = radius * np.stack([np.cos(th), np.sin(th)], axis=1)
    rin = radius * np.cos(np.pi / nb) * (1 - 1e-9)
    u = rng.random(int(n_interior))
    phi = 2 * np.pi * rng.random(int(n_interior))
    rr = rin * np.sqrt(u)
    ipts = np.stack([rr * np.cos(phi), rr * np.sin(phi)], axis=1)
    pts = np.concatenate([bpts, ipts], axis=0)
    seg = list(range(nb)) + [0]
    tri = triangulate_points(pts, boundary_nodes=[seg])
    if tri.num_triangles != 2 * pts.shape[0] - nb - 2:
        raise RuntimeError("disk triangulation is not a triangulation of the boundary polygon")
    return tri
