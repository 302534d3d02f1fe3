"""FVMSystem on the GPU (fvm_system_* through fvmgpu.FVMSystem) against the oracle's system
restatement (oracle/fvm_oracle.py: System, system_fvm_eqs, system_update_dirichlet_nodes):
the right-hand side, the Dirichlet update and Tsit5 solves, on the reference's own system
examples and on a three-component problem that uses every device-coded form."""
import numpy as np
import pytest

import fvm_oracle as O
from fvmgpu.meshes import triangulate_annulus, triangulate_rectangle

pytestmark = pytest.mark.gpu


def _bind(f, p):
    return lambda *a: f(*a, p)


class SysSpec:
    """One system, built for the oracle and for the API from the same closures."""

    def __init__(self, tri, comps, u0, t0=0.0, tf=1.0):
        self.tri, self.comps, self.u0, self.t0, self.tf = tri, comps, u0, t0, tf

    def oracle(self):
        conds, fluxes, sources = [], [], []
        for c in self.comps:
            conds.append(O.Conditions(self.tri, [_bind(f, p) for f, p in zip(c["bc"], c["bcp"])], list(c["types"]),
                                      [_bind(f, p) for f, p in zip(c.get("ic", ()), c.get("icp", ()))],
                                      c.get("dirichlet_nodes"), c.get("dudt_nodes")))
            fluxes.append(_bind(c["q"], c.get("qp")))
            sources.append(_bind(c["S"], c.get("Sp")) if c.get("S") else None)
        return O.System(self.tri, conds, fluxes, sources, u0=self.u0, t0=self.t0, tf=self.tf)

    def api(self, mesh=None):
        import fvmgpu as F

        mesh = mesh or F.FVMGeometry(self.tri)
        probs = []
        for k, c in enumerate(self.comps):
            BCs = F.BoundaryConditions(mesh, tuple(c["bc"]), tuple(getattr(F, t) for t in c["types"]),
                                       parameters=tuple(c["bcp"]))
            ICs = None
            if c.get("ic"):
                ICs = F.InternalConditions(tuple(c["ic"]), dirichlet_nodes=c.get("dirichlet_nodes"),
                                           dudt_nodes=c.get("dudt_nodes"), parameters=tuple(c["icp"]))
            probs.append(F.FVMProblem(mesh, BCs, ICs, flux_function=c["q"], flux_parameters=c.get("qp"),
                                      source_function=c.get("S"), source_parameters=c.get("Sp"),
                                      initial_condition=self.u0[k], initial_time=self.t0, final_time=self.tf))
        return F.FVMSystem(*probs)


def gray_scott(n=30) -> SysSpec:
    """docs/src/literate_tutorials/gray_scott_model_turing_patterns_from_a_coupled_reaction_diffusion_system.jl"""
    tri = triangulate_rectangle(-1.0, 1.0, -1.0, 1.0, n, n, single_boundary=True)
    bc = lambda x, y, t, uv, p: 0.0 * uv[0] * uv[1]  # noqa: E731
    u_q = lambda x, y, t, a, b, g, e1: (-a[0] * e1, -b[0] * e1)  # noqa: E731
    v_q = lambda x, y, t, a, b, g, e2: (-a[1] * e2, -b[1] * e2)  # noqa: E731
    u_S = lambda x, y, t, uv, b: b * (1 - uv[0]) - uv[0] * uv[1] ** 2  # noqa: E731
    v_S = lambda x, y, t, uv, d: -d * uv[1] + uv[0] * uv[1] ** 2  # noqa: E731
    P = tri.points
    r2 = P[:, 0] ** 2 + P[:, 1] ** 2
    u0 = np.stack([1 - np.exp(-80 * r2), np.exp(-80 * r2)])
    comp = lambda q, qp, S, Sp: dict(bc=(bc,), bcp=(None,), types=("Neumann",), q=q, qp=qp, S=S, Sp=Sp)  # noqa: E731
    return SysSpec(tri, [comp(u_q, 0.00002, u_S, 0.04), comp(v_q, 0.00001, v_S, 0.1)], u0, tf=6000.0)


def reference_diffusion_system() -> SysSpec:
    """example_diffusion_problem_system (test/test_functions.jl:318-334)."""
    tri = triangulate_rectangle(0.0, 2.0, 0.0, 2.0, 25, 25, single_boundary=True)
    bc = lambda x, y, t, u, p: 0.0 * u[0] * u[1]  # noqa: E731
    u0 = np.where(tri.points[:, 1] <= 1.0, 50.0, 0.0)
    comps = [dict(bc=(bc,), bcp=(None,), types=("Dirichlet",), q=lambda x, y, t, a, b, g, p: (-a[0] / 9, -b[0] / 9)),
             dict(bc=(bc,), bcp=(None,), types=("Dirichlet",), q=lambda x, y, t, a, b, g, p: (-a[1] / 9, -b[1] / 9))]
    return SysSpec(tri, comps, np.stack([u0, u0]), tf=0.5)


def cross_diffusion_system() -> SysSpec:
    """The reference's diffusion system (test/test_functions.jl:318-334) with a constant
    cross-diffusion matrix [[1/9, 1/20], [1/30, 1/9]]: equal conditions and constant coupled
    blocks, which the library stores as one shared operator."""
    spec = reference_diffusion_system()
    spec.comps[0]["q"] = lambda x, y, t, a, b, g, p: (-(a[0] / 9 + a[1] / 20), -(b[0] / 9 + b[1] / 20))
    spec.comps[1]["q"] = lambda x, y, t, a, b, g, p: (-(a[0] / 30 + a[1] / 9), -(b[0] / 30 + b[1] / 9))
    spec.u0 = spec.u0 * np.array([[1.0], [0.5]])
    return spec


def mixed_system(seed=5) -> SysSpec:
    """Three components on an annulus with eight boundary segments: Dirichlet, Dudt (cubic in
    the components), Neumann (affine in the components, cross-coupled) and Constrained edges,
    internal Dirichlet and Dudt nodes, cross-diffusion fluxes and cubic sources."""
    tri = triangulate_annulus(0.5, 1.0, 9, 48, nsegments=4)
    nseg = tri.num_ghost_vertices
    rng = np.random.default_rng(seed)
    pts = tri.points
    rad = np.linalg.norm(pts, axis=1)
    interior = np.nonzero((rad > 0.6) & (rad < 0.9))[0]
    fd = lambda x, y, t, u, p: x * y - p + 0.0 * x  # noqa: E731
    fdudt = lambda x, y, t, u, p: p * u[0] - u[1] * u[2] + x  # noqa: E731
    fneu = lambda x, y, t, u, p: p * (1.5 - u[1]) + 0.3 * u[0] - y  # noqa: E731
    fneu0 = lambda x, y, t, u, p: 0.0 * x  # noqa: E731
    fcon = lambda x, y, t, u, p: y - x  # noqa: E731
    fdudt3 = lambda x, y, t, u, p: 0.1 * u[2] * u[2] * u[0] - y + p  # noqa: E731
    kinds = {"Dirichlet": (fd, 0.7), "Dudt": (fdudt, 0.3), "Neumann": (fneu, 0.8), "Constrained": (fcon, None)}
    layouts = [("Dirichlet", "Dudt", "Neumann", "Constrained", "Neumann", "Dirichlet", "Dudt", "Neumann"),
               ("Neumann", "Neumann", "Dirichlet", "Neumann", "Dudt", "Neumann", "Neumann", "Dirichlet"),
               ("Neumann",) * 8]
    fluxes = [lambda x, y, t, a, b, g, p: (-((1 + x * x) * a[0] + 0.1 * a[1]), -((1 + x * x) * b[0] + 0.1 * b[1])),
              lambda x, y, t, a, b, g, p: (-(0.5 * a[1] - 0.2 * y * a[2]), -(0.5 * b[1] - 0.2 * y * b[2])),
              lambda x, y, t, a, b, g, p: (-p * a[2], -p * b[2])]
    sources = [lambda x, y, t, u, p: u[0] * u[1] - u[2] ** 2 + x,
               lambda x, y, t, u, p: p * u[0] ** 2 * u[2] - u[1],
               lambda x, y, t, u, p: -u[0] + 2.0 * u[1] * u[2] * u[0] + 0.0 * x]
    comps = []
    for k, lay in enumerate(layouts[:3]):
        lay = lay[:nseg]
        bc, bcp = [], []
        for s, typ in enumerate(lay):
            f, p = kinds[typ]
            if typ == "Dudt" and k == 1:
                f, p = fdudt3, 0.2
            if typ == "Neumann" and s % 3 == 2:
                f, p = fneu0, None
            bc.append(f)
            bcp.append(p)
        c = dict(bc=tuple(bc), bcp=tuple(bcp), types=lay, q=fluxes[k], qp=0.9 if k == 2 else None, S=sources[k],
                 Sp=0.3 if k == 1 else None)
        if k == 1:
            c.update(ic=(lambda x, y, t, u, p: x + y + p + 0.0 * x,), icp=(0.29,),
                     dirichlet_nodes={int(interior[3]): 0})
        if k == 2:
            c.update(ic=(lambda x, y, t, u, p: -0.5 * u[2] + p * u[0] * u[1],), icp=(0.1,),
                     dudt_nodes={int(interior[11]): 0})
        comps.append(c)
    u0 = rng.standard_normal((3, tri.num_points))
    return SysSpec(tri, comps, u0, tf=0.1)


def brusselator(n=100, tf=5.0) -> SysSpec:
    """The Brusselator tutorial (docs/src/literate_tutorials/reaction_diffusion_brusselator_system_of_pdes.jl:84-124):
    unit square, fluxes -grad(Phi)/4 and -grad(Psi)/4, sources Phi^2 Psi - 2 Phi and
    -Phi^2 Psi + Phi, boundary values with factors exp(-t/2) and exp(t/2).  Its exact solution
    is Phi = exp(-x - y - t/2), Psi = exp(x + y + t/2)."""
    tri = triangulate_rectangle(0.0, 1.0, 0.0, 1.0, n, n, single_boundary=False)
    phi_bc = (lambda x, y, t, u, p: -1 / 4 * np.exp(-x - t / 2), lambda x, y, t, u, p: 1 / 4 * np.exp(-1 - y - t / 2),
              lambda x, y, t, u, p: np.exp(-1 - x - t / 2), lambda x, y, t, u, p: -1 / 4 * np.exp(-y - t / 2))
    psi_bc = (lambda x, y, t, u, p: np.exp(x + t / 2), lambda x, y, t, u, p: -1 / 4 * np.exp(1 + y + t / 2),
              lambda x, y, t, u, p: -1 / 4 * np.exp(1 + x + t / 2), lambda x, y, t, u, p: np.exp(y + t / 2))
    P = tri.points
    comps = [dict(bc=phi_bc, bcp=(None,) * 4, types=("Neumann", "Neumann", "Dirichlet", "Neumann"),
                  q=lambda x, y, t, a, b, g, p: (-a[0] / 4, -b[0] / 4),
                  S=lambda x, y, t, u, p: u[0] ** 2 * u[1] - 2 * u[0]),
             dict(bc=psi_bc, bcp=(None,) * 4, types=("Dirichlet", "Neumann", "Neumann", "Dirichlet"),
                  q=lambda x, y, t, a, b, g, p: (-a[1] / 4, -b[1] / 4),
                  S=lambda x, y, t, u, p: -u[0] ** 2 * u[1] + u[0])]
    u0 = np.stack([np.exp(-P[:, 0] - P[:, 1]), np.exp(P[:, 0] + P[:, 1])])
    return SysSpec(tri, comps, u0, tf=tf)


def brusselator_exact(P, t):
    return np.stack([np.exp(-P[:, 0] - P[:, 1] - t / 2), np.exp(P[:, 0] + P[:, 1] + t / 2)])


def _rhs_close(got, ref, tol=1e-12):
    for c in range(ref.shape[0]):
        assert np.max(np.abs(got[c] - ref[c])) <= tol * np.max(np.abs(ref[c])), c


@pytest.mark.parametrize("make", [gray_scott, reference_diffusion_system, cross_diffusion_system, mixed_system])
def test_system_rhs_matches_oracle(gpu_lib, make):
    spec = make()
    osys, sys = spec.oracle(), spec.api()
    rng = np.random.default_rng(8)
    for u in (spec.u0, rng.standard_normal(spec.u0.shape) + 0.5):
        ref = O.system_fvm_eqs(osys, u, 0.0)
        got = np.empty_like(u)
        sys.rhs(got, u, 0.0)
        _rhs_close(got, ref)
    # conditions read back exactly: rows without a condition are the free ones, in the oracle's order
    assert np.array_equal(sys._codes, osys.code)


def test_system_forms_and_info(gpu_lib):
    sys = gray_scott().api()
    info = sys.info()
    # diagonal coupling: the two stored blocks issue fewer FP64 FMAs than a shared operator would
    assert info == {"neqs": 2, "flux_blocks": 2, "terms": 5, "varying_terms": 0, "dirichlet_entries": 0,
                    "has_neumann_constants": 0, "shared_operator": 0}
    ci = cross_diffusion_system().api().info()
    assert ci["flux_blocks"] == 4 and ci["shared_operator"] == 1 and ci["dirichlet_entries"] > 0
    msys = mixed_system().api()
    mi = msys.info()
    assert mi["neqs"] == 3 and mi["flux_blocks"] == 8 and mi["dirichlet_entries"] > 0 and mi["has_neumann_constants"]
    assert not mi["shared_operator"] and mi["terms"] == 13


def test_system_dirichlet_update_matches_oracle(gpu_lib):
    import fvmgpu as F

    spec = mixed_system()
    osys, sys = spec.oracle(), spec.api()
    u = spec.u0.copy()
    F.update_dirichlet_nodes(u, sys, 0.0)
    assert np.array_equal(u, O.system_update_dirichlet_nodes(osys, spec.u0, 0.0))


def test_system_device_tensors_match_host(gpu_lib):
    import torch
    import fvmgpu as F

    spec = mixed_system()
    sys = spec.api()
    n = spec.tri.num_points
    u = spec.u0
    ref = np.empty_like(u)
    F.fvm_eqs(ref, u, sys, 0.0)
    ud = torch.from_numpy(np.ascontiguousarray(u.T)).cuda().T  # (N, n) view of [point][component] memory
    dud = torch.empty((n, 3), dtype=torch.float64, device="cuda").T
    F.fvm_eqs(dud, ud, sys, 0.0)
    torch.cuda.synchronize()
    assert np.array_equal(dud.cpu().numpy(), ref)


def test_reference_diffusion_system_solves_like_single_problem(gpu_lib):
    """test/equations.jl:106-121: both components of the system equal the single problem."""
    import fvmgpu as F
    from problems import api_problem, readme_diffusion

    spec = reference_diffusion_system()
    sys = spec.api()
    prob = api_problem(readme_diffusion(25), mesh=sys.mesh)
    sols = F.solve(sys, F.Tsit5(), saveat=0.05)
    solp = F.solve(prob, F.Tsit5(), saveat=0.05)
    assert len(sols.u) == len(solp.u) == 11 and sols.u[3].shape == (2, spec.tri.num_points)
    # the single problem runs on the cluster driver, the system on the graph-looped one: equal
    # step control up to last-bit differences, solutions within the reference test's isapprox
    for us, up in zip(sols.u, solp.u):
        for c in range(2):
            assert np.max(np.abs(us[c] - up)) <= 1e-8 * 50
    assert abs(sols.stats["naccept"] - solp.stats["naccept"]) <= 1


@pytest.mark.parametrize("adaptive", [False, True])
def test_system_tsit5_matches_oracle(gpu_lib, adaptive):
    import fvmgpu as F

    spec = mixed_system()
    spec.tf = 0.02
    osys, sys = spec.oracle(), spec.api()
    f = lambda v, t: O.system_fvm_eqs(osys, v, t)  # noqa: E731
    cb = lambda v, t: O.system_update_dirichlet_nodes(osys, v, t)  # noqa: E731
    ts = np.linspace(0.0, 0.02, 5)
    if adaptive:
        sol = F.solve(sys, F.Tsit5(), saveat=ts, abstol=1e-8, reltol=1e-6)
        ref, st = O.tsit5_solve(f, spec.u0, 0.0, 0.02, ts, abstol=1e-8, reltol=1e-6, callback=cb)
        tol = 1e-8
        assert sol.stats["naccept"] == st["naccept"]
    else:
        sol = F.solve(sys, F.Tsit5(), saveat=ts, dt=2e-4, adaptive=False)
        ref, _ = O.tsit5_solve(f, spec.u0, 0.0, 0.02, ts, dt=2e-4, adaptive=False, callback=cb)
        tol = 1e-10
    got = np.array(sol.u)
    assert np.max(np.abs(got - ref)) <= tol * np.max(np.abs(ref))


def test_gray_scott_tutorial_size_rhs_and_steps(gpu_lib):
    """The tutorial's 200 x 200 mesh: RHS parity at its initial condition and a short fixed-step
    run against the oracle."""
    import fvmgpu as F

    spec = gray_scott(200)
    osys, sys = spec.oracle(), spec.api()
    got = np.empty_like(spec.u0)
    sys.rhs(got, spec.u0)
    _rhs_close(got, O.system_fvm_eqs(osys, spec.u0, 0.0))
    sol = F.solve(sys, F.Tsit5(), saveat=[0.0, 20.0], dt=1.0, adaptive=False)
    ref, _ = O.tsit5_solve(lambda v, t: O.system_fvm_eqs(osys, v, t), spec.u0, 0.0, 20.0, [0.0, 20.0], dt=1.0,
                           adaptive=False)
    assert np.max(np.abs(sol.u[-1] - ref[-1])) <= 1e-11


def test_system_errors(gpu_lib):
    import fvmgpu as F

    spec = gray_scott(10)
    mesh = F.FVMGeometry(spec.tri)
    BCs = F.BoundaryConditions(mesh, (lambda x, y, t, u, p: 0.0 * x,), (F.Neumann,))
    pD = F.FVMProblem(mesh, BCs, diffusion_function=lambda x, y, t, u, p: 1.0 + 0.0 * x,
                      initial_condition=spec.u0[0], final_time=1.0)
    with pytest.raises(F.InvalidFluxError):  # test/equations.jl:108
        F.FVMSystem(pD, pD)
    q = lambda x, y, t, a, b, g, p: (-a[0], -b[0])  # noqa: E731
    p1 = F.FVMProblem(mesh, BCs, flux_function=q, initial_condition=spec.u0[0], final_time=1.0)
    p2 = F.FVMProblem(mesh, BCs, flux_function=q, initial_condition=spec.u0[1], final_time=2.0)
    with pytest.raises(AssertionError):
        F.FVMSystem(p1, p2)
    with pytest.raises(ValueError):
        F.FVMSystem()
    # exp(-x - t/2) is a device form (a time factor); sin(3t) is not
    tdep = F.BoundaryConditions(mesh, (lambda x, y, t, u, p: np.sin(3 * t) * np.exp(-x),), (F.Neumann,))
    p3 = F.FVMProblem(mesh, tdep, flux_function=q, initial_condition=spec.u0[0], final_time=1.0)
    with pytest.raises(F.UnsupportedFormError):
        F.FVMSystem(p3, p1)
    p4 = F.FVMProblem(mesh, BCs, flux_function=q, source_function=lambda x, y, t, u, p: np.sin(u[0]),
                      initial_condition=spec.u0[0], final_time=1.0)
    with pytest.raises(F.UnsupportedFormError):
        F.FVMSystem(p4, p1)


@pytest.mark.parametrize("N", [2, 5])
def test_system_rolled_kernel_on_wide_rows(gpu_lib, N):
    """A hub vertex of degree 40 (rows wider than 16 slots) and five components take the kernel's
    rolled slot loop; two components with coupled constant blocks take its shared form."""
    from problems import wheel_mesh

    tri = wheel_mesh(40)
    rng = np.random.default_rng(9)
    P = tri.points
    if N == 2:  # constant coupled blocks, equal conditions: the shared form
        q = [lambda x, y, t, a, b, g, p: (-(a[0] + 0.2 * a[1]), -(b[0] + 0.2 * b[1])),
             lambda x, y, t, a, b, g, p: (-(0.1 * a[0] + 0.5 * a[1]), -(0.1 * b[0] + 0.5 * b[1]))]
        S = [lambda x, y, t, u, p: u[0] * u[1] - x, lambda x, y, t, u, p: -u[1] ** 3 + 0.0 * x]
    else:
        q = [(lambda c: lambda x, y, t, a, b, g, p: (-(1 + x * x) * a[c] - 0.1 * a[(c + 1) % 5],
                                                   -(1 + x * x) * b[c] - 0.1 * b[(c + 1) % 5]))(c) for c in range(5)]
        S = [(lambda c: lambda x, y, t, u, p: u[c] * u[(c + 2) % 5] - 0.5 * u[c] + y)(c) for c in range(5)]
    if N == 2:  # a Neumann value independent of u keeps the blocks shareable
        bc = lambda x, y, t, u, p: 0.3 - x  # noqa: E731
    else:
        bc = lambda x, y, t, u, p: 0.5 * u[0] - x  # noqa: E731
    comps = [dict(bc=(bc,), bcp=(None,), types=("Neumann",), q=q[c], S=S[c]) for c in range(N)]
    spec = SysSpec(tri, comps, rng.standard_normal((N, tri.num_points)), tf=0.1)
    osys, sys = spec.oracle(), spec.api()
    assert sys.mesh.info()["operator_slots"] > 0
    assert sys.info()["shared_operator"] == (1 if N == 2 else 0)
    for u in (spec.u0, rng.standard_normal(spec.u0.shape)):
        got = np.empty_like(u)
        sys.rhs(got, u, 0.0)
        _rhs_close(got, O.system_fvm_eqs(osys, u, 0.0))


def test_brusselator_rhs_and_dirichlet_at_any_t(gpu_lib):
    """The Brusselator's time-dependent boundary values (two factors, exp(-t/2) and exp(t/2),
    on Neumann and Dirichlet edges of both components): RHS and Dirichlet update against the
    oracle at times inside and beyond the time span."""
    import fvmgpu as F

    spec = brusselator(30)
    osys, sys = spec.oracle(), spec.api()
    assert sorted(round(f[2], 9) for f in sys.time_factors) == [-0.5, 0.5]
    rng = np.random.default_rng(4)
    u = spec.u0 * (1 + 0.1 * rng.standard_normal(spec.u0.shape))
    for t in (0.0, 0.7, 5.0, 7.5):
        got = np.empty_like(u)
        sys.rhs(got, u, t)
        _rhs_close(got, O.system_fvm_eqs(osys, u, t))
        v = u.copy()
        F.update_dirichlet_nodes(v, sys, t)
        w = O.system_update_dirichlet_nodes(osys, u, t)
        assert np.max(np.abs(v - w)) <= 1e-14 * np.max(np.abs(w)), t


def test_brusselator_solve_matches_oracle(gpu_lib):
    """Adaptive Tsit5 on a 16 x 16 Brusselator to t = 0.3 against the oracle's driver: the
    host-controlled loop, the same steps, snapshots within 1e-8 of max|u|."""
    import fvmgpu as F

    spec = brusselator(16, tf=0.3)
    osys, sys = spec.oracle(), spec.api()
    ts = np.linspace(0.0, 0.3, 7)
    sol = F.solve(sys, F.Tsit5(), saveat=ts, abstol=1e-8, reltol=1e-6)
    ref, st = O.tsit5_solve(lambda v, t: O.system_fvm_eqs(osys, v, t), spec.u0, 0.0, 0.3, ts, abstol=1e-8,
                            reltol=1e-6, callback=lambda v, t: O.system_update_dirichlet_nodes(osys, v, t))
    assert sol.stats["driver"] == "host"
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    assert sol.stats["nrhs"] == st["nrhs"]
    got = np.array(sol.u)
    assert np.max(np.abs(got - ref)) <= 1e-8 * np.max(np.abs(ref))


def test_brusselator_tutorial_mesh_converges_to_exact_solution(gpu_lib):
    """The tutorial's 100 x 100 mesh (and 50 x 50) to t = 1: the GPU solution is within the
    discretisation error of the exact solution, which falls with h."""
    import fvmgpu as F

    errs = []
    for n in (50, 100):
        spec = brusselator(n, tf=1.0)
        sys = spec.api()
        sol = F.solve(sys, F.Tsit5(), saveat=[1.0], abstol=1e-9, reltol=1e-9)
        ex = brusselator_exact(spec.tri.points, 1.0)
        errs.append(max(np.max(np.abs(sol.u[-1][c] - ex[c])) / np.max(ex[c]) for c in range(2)))
    assert errs[1] < 1e-3 and errs[1] < 0.5 * errs[0], errs


def _flat_oracle(osys, N):
    """The oracle's system fvm_eqs! on states flattened [point][component] (the numbering of
    jacobian_sparsity(tri, N): node i's unknowns i N + l)."""
    return lambda x, t: O.system_fvm_eqs(osys, x.reshape(-1, N).T, t).T.ravel()


@pytest.mark.parametrize("make", [lambda: gray_scott(12), mixed_system, lambda: brusselator(10),
                                  cross_diffusion_system])
def test_system_jvp_and_diagonal_against_oracle(gpu_lib, make):
    """J(u) v of the system (block operator plus the polynomial derivatives, stored and shared
    block forms) against central differences of the oracle's system fvm_eqs!, and diag J
    against the oracle's coloured finite-difference Jacobian."""
    import torch

    import fvmgpu as F

    spec = make()
    osys, sys = spec.oracle(), spec.api()
    N, n = spec.u0.shape
    rng = np.random.default_rng(11)
    u = spec.u0 + 0.1 * rng.standard_normal(spec.u0.shape)
    v = rng.standard_normal(spec.u0.shape)
    t = 0.3
    got = F.jvp(sys, u, v, t)
    eps = 1e-5
    fd = (O.system_fvm_eqs(osys, u + eps * v, t) - O.system_fvm_eqs(osys, u - eps * v, t)) / (2 * eps)
    assert np.max(np.abs(got - fd)) <= 1e-7 * np.max(np.abs(fd))
    dev = lambda a: torch.tensor(np.ascontiguousarray(a.T), device="cuda").T  # noqa: E731
    got_d = F.jvp(sys, dev(u), dev(v), t)
    assert np.array_equal(got_d.cpu().numpy(), got)
    ent, nn = O.jacobian_sparsity(spec.tri, N)
    J = O.colored_jacobian(_flat_oracle(osys, N), u.T.ravel(), t, ent, nn)
    want = J.diagonal().reshape(n, N).T
    diag = F.jacobian_diagonal(sys, u, t)
    assert np.max(np.abs(diag - want)) <= 1e-6 * np.max(np.abs(want))


def _oracle_system_trbdf2(spec, saveat, **kw):
    osys = spec.oracle()
    N = spec.u0.shape[0]
    f = _flat_oracle(osys, N)
    ent, nn = O.jacobian_sparsity(spec.tri, N)
    jac = lambda x, t: O.colored_jacobian(f, x, t, ent, nn)  # noqa: E731
    cb = lambda x, t: O.system_update_dirichlet_nodes(osys, x.reshape(-1, N).T, t).T.ravel()  # noqa: E731
    ref, st = O.trbdf2_solve(f, jac, spec.u0.T.ravel(), spec.t0, spec.tf, saveat, callback=cb, **kw)
    return np.array([r.reshape(-1, N).T for r in ref]), st


def test_system_trbdf2_matches_oracle(gpu_lib):
    """TR-BDF2 on a 12 x 12 Brusselator (nonlinear sources, time-dependent Dirichlet and Neumann
    values) to t = 0.2 at tight tolerances: Newton with the exact device JVP against the
    oracle's with a finite-difference Jacobian and exact sparse solves."""
    import fvmgpu as F

    spec = brusselator(12, tf=0.2)
    sys = spec.api()
    saveat = [0.0, 0.1, 0.2]
    sol = F.solve(sys, F.TRBDF2(), saveat=saveat, abstol=1e-8, reltol=1e-8)
    ref, st = _oracle_system_trbdf2(spec, saveat, abstol=1e-8, reltol=1e-8)
    assert abs(sol.stats["naccept"] - st["naccept"]) <= 2
    got = np.array(sol.u)
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref))


def test_system_trbdf2_mixed_forms_fixed_step(gpu_lib):
    """Fixed-step TR-BDF2 on the three-component system with every device-coded form (Dudt
    and Neumann boundaries coupled across components, internal Dirichlet and Dudt nodes, cubic
    sources): the oracle's steps, 1e-7 of max|u|."""
    import fvmgpu as F

    spec = mixed_system()
    spec.tf = 0.01
    sys = spec.api()
    saveat = [0.0, 0.005, 0.01]
    sol = F.solve(sys, F.TRBDF2(), saveat=saveat, dt=1e-3, adaptive=False)
    ref, st = _oracle_system_trbdf2(spec, saveat, dt=1e-3, adaptive=False)
    assert sol.stats["naccept"] == st["naccept"] == 10
    got = np.array(sol.u)
    assert np.max(np.abs(got - ref)) <= 1e-7 * np.max(np.abs(ref))


def test_system_trbdf2_affine_takes_one_newton_iteration(gpu_lib):
    """A system with no product of components (the cross-diffusion system) is affine: one
    Newton iteration per stage, and the oracle's steps."""
    import fvmgpu as F

    spec = cross_diffusion_system()
    spec.tf = 0.05
    sys = spec.api()
    saveat = [0.0, 0.05]
    sol = F.solve(sys, F.TRBDF2(), saveat=saveat)
    ref, st = _oracle_system_trbdf2(spec, saveat, affine=True)
    assert sol.stats["naccept"] == st["naccept"]
    assert sol.stats["newton_iters"] == 2 * (sol.stats["naccept"] + sol.stats["nreject"])
    got = np.array(sol.u)
    assert np.max(np.abs(got - ref)) <= 1e-8 * np.max(np.abs(ref))


def test_brusselator_tutorial_trbdf2(gpu_lib):
    """The tutorial's call, solve(system, TRBDF2(), saveat = 1.0) on the 100 x 100 mesh to t = 5:
    A-stable steps set by accuracy, not the diffusion limit (measured 363 against Tsit5's
    28,988), and the exact solution within the integration tolerance (largest relative error
    over the saves measured 9.7e-3; default-tolerance Tsit5 on the same mesh: 2.8e-2)."""
    import fvmgpu as F

    spec = brusselator(100, tf=5.0)
    sys = spec.api()
    saveat = np.arange(0.0, 5.0 + 1e-12, 1.0)
    sol = F.solve(sys, F.TRBDF2(), saveat=saveat)
    assert sol.stats["naccept"] < 500
    for k, t in enumerate(saveat):
        ex = brusselator_exact(spec.tri.points, t)
        err = max(np.max(np.abs(sol.u[k][c] - ex[c])) / np.max(ex[c]) for c in range(2))
        assert err < 2e-2, (t, err)
