"""The device mesh build (fvm_mesh_create's default) against the host build
(FVM_MESH_HOST_INGEST): control volumes, triangle properties, Hilbert order, operator pattern,
boundary elements and a right-hand side, all bit-identical; mesh errors reported alike."""
import numpy as np
import pytest

from fvmgpu.meshes import Triangulation, triangulate_annulus, triangulate_disk, triangulate_rectangle
from problems import api_problem, sine_diffusion, wheel_mesh

pytestmark = pytest.mark.gpu


def _with_orphan_points(tri):
    """The same mesh with two extra points in no triangle (the reference allows them)."""
    pts = np.vstack([tri.points, [[0.123, 0.456], [0.789, 0.012]]])
    return Triangulation(pts, tri.triangles, tri.boundary_nodes)


MESHES = {
    "rectangle": lambda: triangulate_rectangle(0.0, 2.0, 0.0, 1.0, 37, 23, single_boundary=False),
    "annulus": lambda: triangulate_annulus(0.5, 1.0, 9, 48, nsegments=4),
    "disk": lambda: triangulate_disk(5000, 200, seed=3),
    "wheel": lambda: wheel_mesh(40),
    "orphans": lambda: _with_orphan_points(triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 12, 12)),
}


def _mesh_data(mesh):
    cv, props = mesh.cv_volumes, mesh.props_array
    perm = mesh.permutation()
    info = mesh.info()
    tris, belems = mesh.export_connectivity()
    return cv, props, perm, info, tris, belems


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("renumber", [True, False])
def test_device_ingest_matches_host(gpu_lib, name, renumber):
    import fvmgpu as F

    tri = MESHES[name]()
    dev = F.FVMGeometry(tri, renumber=renumber)
    host = F.FVMGeometry(tri, renumber=renumber, host_ingest=True)
    for a, b in zip(_mesh_data(dev), _mesh_data(host)):
        if isinstance(a, dict):
            assert a == b
        else:
            assert np.array_equal(a, b)


def test_device_ingest_rhs_bit_identical_at_1m_points(gpu_lib):
    """The 1000 x 1000 mesh of the benchmarked RHS: the same operator, so the same RHS bits."""
    import fvmgpu as F

    spec = sine_diffusion(1000)
    dev = F.FVMGeometry(spec.tri)
    host = F.FVMGeometry(spec.tri, host_ingest=True)
    assert np.array_equal(dev.cv_volumes, host.cv_volumes)
    assert np.array_equal(dev.props_array, host.props_array)
    assert np.array_equal(dev.permutation(), host.permutation())
    u = spec.u0 + np.random.default_rng(2).standard_normal(spec.tri.num_points)
    outs = []
    for mesh in (dev, host):
        prob = api_problem(spec, mesh=mesh)
        outs.append(F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0))
    assert np.array_equal(outs[0], outs[1])


def _create_status(points, tris, be, badj, flags):
    """fvm_mesh_create through the C ABI: (status, last error text)."""
    import ctypes as C

    from fvmgpu import _lib

    lib = _lib.load()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    t = np.ascontiguousarray(tris, dtype=np.int32)
    b = np.ascontiguousarray(be, dtype=np.int32)
    a = None if badj is None else np.ascontiguousarray(badj, dtype=np.int32)
    h = C.c_void_p()
    st = lib.fvm_mesh_create(_lib.dptr(pts), pts.shape[0], _lib.dptr(t, _lib.c_int32_p), t.shape[0],
                             _lib.dptr(b, _lib.c_int32_p), None if a is None else _lib.dptr(a, _lib.c_int32_p),
                             b.shape[0], 0, flags, C.byref(h))
    buf = C.create_string_buffer(512)
    lib.fvm_last_error(buf, 512)
    if st == 0:
        lib.fvm_mesh_destroy(h)
    return st, buf.value.decode()


def test_device_ingest_reports_bad_meshes(gpu_lib):
    """A clockwise triangle, a boundary edge with no triangle on its left and a wrong
    boundary_adjacent entry: FVM_ERR_BAD_MESH with the host build's message."""
    from fvmgpu import _lib

    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 6, 6)
    P, T, BE, BA = tri.points, tri.triangles, tri.boundary_edges, tri.boundary_adjacent
    bad = T.copy()
    bad[7] = bad[7][[0, 2, 1]]  # clockwise
    (i, j), k = BE[3], BA[3]
    holed = T[[set(map(int, t)) != {int(i), int(j), int(k)} for t in T]]
    wrong = BA.copy()
    wrong[5] = wrong[6]
    cases = [(bad, BA, "triangle 7 is clockwise"), (holed, None, "boundary edge 3"),
             (T, wrong, "boundary_adjacent[5]")]
    for tris, adj, what in cases:
        res = [_create_status(P, tris, BE, adj, f) for f in (0, _lib.FVM_MESH_HOST_INGEST)]
        assert res[0][0] == res[1][0] == _lib.FVM_ERR_BAD_MESH, res
        assert res[0][1] == res[1][1] and what in res[0][1], res
