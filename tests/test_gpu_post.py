"""Post-processing on the device: point location (fvm_mesh_locate) against a brute-force
search, and pl_interpolate for many points (fvm_pl_interpolate) against the reference's formula
(src/utils.jl:23-27) evaluated on the host -- bit-identical, the device code has no FMA
contraction -- for scalar problems and systems, host arrays, device tensors and the internal
numbering."""
import numpy as np
import pytest

from fvmgpu.meshes import triangulate_annulus, triangulate_disk, triangulate_rectangle

pytestmark = pytest.mark.gpu


def _containing(tri, xy):
    """Per point, the sorted list of triangles containing it (orientation tests >= -tol)."""
    P, T = tri.points, tri.triangles
    a, b, c = P[T[:, 0]], P[T[:, 1]], P[T[:, 2]]
    out = []
    for px, py in xy:
        def orient(u, v):
            return (v[:, 0] - u[:, 0]) * (py - u[:, 1]) - (v[:, 1] - u[:, 1]) * (px - u[:, 0])
        area = np.abs(orient(a, b) * 0 + ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])))
        m = np.minimum(np.minimum(orient(a, b), orient(b, c)), orient(c, a)) / area
        out.append(np.nonzero(m >= -1e-12)[0])
    return out


def _host_interp(mesh, t, u, x, y):
    """The reference's formula with the stored shape coefficients, in its operation order."""
    T = mesh.triangulation.triangles[t]
    s = mesh.props_array[t, :9]
    ua, ub, uc = u[..., T[:, 0]], u[..., T[:, 1]], u[..., T[:, 2]]
    al = s[:, 0] * ua + s[:, 1] * ub + s[:, 2] * uc
    be = s[:, 3] * ua + s[:, 4] * ub + s[:, 5] * uc
    ga = s[:, 6] * ua + s[:, 7] * ub + s[:, 8] * uc
    return al * x + be * y + ga


@pytest.mark.parametrize("make", [lambda: triangulate_disk(3000, 128, seed=4),
                                  lambda: triangulate_annulus(0.2, 1.0, 12, 64, nsegments=2)])
def test_locate_against_brute_force(gpu_lib, make):
    import fvmgpu as F

    tri = make()
    mesh = F.FVMGeometry(tri)
    rng = np.random.default_rng(5)
    xy = rng.uniform(-1.1, 1.1, size=(3000, 2))
    xy = np.vstack([xy, tri.points[:200]])  # vertices: on several triangles at once
    got = mesh.locate(xy)
    want = _containing(tri, xy)
    for q, (g, w) in enumerate(zip(got, want)):
        if w.size == 0:
            assert g == -1, q
        else:
            assert g in w and g == w.min(), (q, g, w)


def test_interpolate_matches_reference_formula(gpu_lib):
    import torch
    import fvmgpu as F

    tri = triangulate_rectangle(0.0, 2.0, -1.0, 1.0, 80, 60)
    mesh = F.FVMGeometry(tri)
    rng = np.random.default_rng(6)
    P = tri.points
    u = np.sin(3 * P[:, 0]) * np.cos(2 * P[:, 1]) + 0.1 * rng.standard_normal(tri.num_points)
    x = rng.uniform(-0.1, 2.1, 5000)
    y = rng.uniform(-1.1, 1.1, 5000)
    got = F.interpolate(mesh, u, x, y)
    t = mesh.locate(x, y)
    inside = t >= 0
    assert np.all(np.isnan(got[~inside])) and inside.sum() > 4000
    assert np.array_equal(got[inside], _host_interp(mesh, t[inside], u, x[inside], y[inside]))
    # the scalar pl_interpolate on a few points agrees exactly
    for q in np.nonzero(inside)[0][:20]:
        assert F.pl_interpolate(mesh_prob(F, mesh, u), tuple(tri.triangles[t[q]]), u, x[q], y[q]) == got[q]
    # systems: (N, npoints) u gives (N, nq)
    U = np.stack([u, 2 * u + 1, P[:, 0]])
    G = F.interpolate(mesh, U, x, y, T=t)
    assert G.shape == (3, 5000)
    assert np.array_equal(G[:, inside], _host_interp(mesh, t[inside], U, x[inside], y[inside]))
    assert np.allclose(G[2, inside], x[inside], rtol=0, atol=1e-12)  # linear fields are reproduced
    # device tensors, and u in the library's internal numbering
    xy_d = torch.as_tensor(np.stack([x, y], axis=1), device="cuda")
    u_d = torch.as_tensor(u, device="cuda")
    got_d = F.interpolate(mesh, u_d, xy_d)
    assert torch.equal(torch.isnan(got_d).cpu(), torch.as_tensor(~inside))
    assert np.array_equal(got_d.cpu().numpy()[inside], got[inside])


def mesh_prob(F, mesh, u):
    """A minimal problem on the mesh (pl_interpolate takes a problem, as the reference's does)."""
    BCs = F.BoundaryConditions(mesh, (lambda x, y, t, u, p: 0.0 * x,) * mesh.triangulation.num_ghost_vertices,
                               (F.Dirichlet,) * mesh.triangulation.num_ghost_vertices)
    return F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x, initial_condition=u,
                        final_time=1.0)


def test_interpolate_tutorial_grid_on_the_annulus(gpu_lib):
    """The annulus tutorial's post-processing: u on a 400 x 400 grid of [-1, 1]^2, NaN where the
    grid point lies outside the mesh (the hole and the corners), values within the range of u."""
    import fvmgpu as F

    tri = triangulate_annulus(0.2, 1.0, 24, 96, nsegments=1)
    mesh = F.FVMGeometry(tri)
    P = tri.points
    u = 10 * np.exp(-25 * ((P[:, 0] + 0.5) ** 2 + (P[:, 1] + 0.5) ** 2))
    g = np.linspace(-1, 1, 400)
    X, Y = np.meshgrid(g, g, indexing="ij")
    V = F.interpolate(mesh, u, X.ravel(), Y.ravel()).reshape(400, 400)
    r = np.hypot(X, Y)
    assert np.all(np.isnan(V[(r > 1.0 + 1e-9) | (r < 0.19)]))
    inner = (r < 0.97) & (r > 0.25)  # inside the polygonal annulus
    assert np.all(np.isfinite(V[inner])) and np.nanmin(V) >= u.min() - 1e-12 and np.nanmax(V) <= u.max() + 1e-12
