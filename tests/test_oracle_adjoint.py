"""CPU checks of the oracle pieces the adjoint tests rest on: the P1 interpolant of vertex
values (exact on linear fields, scalar and array queries) and the template assembly with a
P1 diffusion field (A's rows sum to zero on interior vertices: constant fields carry no flux)."""
import numpy as np

import fvm_oracle as O
from fvmgpu.meshes import triangulate_rectangle


def test_p1_field_is_exact_on_linear_fields():
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 7, 5, single_boundary=True)
    v = 3 * tri.points[:, 0] - 2 * tri.points[:, 1] + 1
    f = O.p1_field(tri, v)
    rng = np.random.default_rng(0)
    x, y = rng.random(40), rng.random(40)
    assert np.max(np.abs(f(x, y) - (3 * x - 2 * y + 1))) < 1e-14
    assert isinstance(f(0.25, 0.0), float) and abs(f(0.25, 0.0) - 1.75) < 1e-14
    assert f(x.reshape(5, 8), y.reshape(5, 8)).shape == (5, 8)


def test_template_with_p1_diffusion_conserves_constants():
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, 9, 9, single_boundary=True)
    theta = 0.3 * np.sin(3 * tri.points[:, 0]) * np.cos(2 * tri.points[:, 1])
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b, _ = O.template_diffusion(tri, conds, O.p1_field(tri, np.exp(theta)), np.zeros(tri.num_points))
    rows = np.asarray(A.sum(axis=1)).ravel()
    scale = np.asarray(abs(A).sum(axis=1)).ravel()
    assert np.all(np.abs(rows) <= 1e-13 * np.maximum(scale, 1.0))
    assert np.count_nonzero(A.diagonal()) == (7 * 7)  # interior rows only: Dirichlet rows are zero
