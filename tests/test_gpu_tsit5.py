"""GPU Tsit5 (fixed step, CUDA-graph replay, adaptive PI control with saveat) against the
oracle's Tsit5 driver, which restates the same step control.  Tolerance: 1e-10 relative to
max|u| for fixed steps, 1e-8 for adaptive runs (identical step sequences, rounding only)."""
import numpy as np
import pytest

import fvm_oracle as O
from problems import (api_problem, mixed_annulus, nonlinear_rect, oracle_problem, readme_diffusion, sine_diffusion,
                      wheel_diffusion)

pytestmark = pytest.mark.gpu


def _oracle_run(spec, saveat, dt=None, adaptive=True):
    prob = oracle_problem(spec)
    cb = (lambda u, t: O.update_dirichlet_nodes(prob, u, t)) if prob.conds.dirichlet_nodes else None
    return O.tsit5_solve(lambda u, t: O.fvm_eqs(prob, u, t), spec.u0, spec.t0, spec.tf, saveat, dt=dt,
                         adaptive=adaptive, callback=cb)


@pytest.mark.parametrize("use_graph", [True, False])
def test_fixed_step_tsit5(gpu_lib, use_graph):
    import fvmgpu as F

    spec = sine_diffusion(32)
    spec.tf = 2e-3
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), dt=1e-4, adaptive=False, saveat=[spec.tf], use_graph=use_graph)
    ref, st = _oracle_run(spec, [spec.tf], dt=1e-4, adaptive=False)
    err = np.max(np.abs(sol.u[-1] - ref[-1])) / np.max(np.abs(ref[-1]))
    assert err < 1e-10, err
    assert sol.stats["naccept"] == st["naccept"] == 20


def test_fixed_step_dense_output(gpu_lib):
    """saveat points inside fixed steps (dt = 3.7e-4, saves every 1e-3): Tsit5's continuous
    extension on the GPU against the oracle's, 1e-10 of max|u|."""
    import fvmgpu as F

    spec = readme_diffusion(50)
    spec.tf = 0.05
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), dt=3.7e-4, adaptive=False, saveat=0.001)
    ref, st = _oracle_run(spec, list(sol.t), dt=3.7e-4, adaptive=False)
    assert len(sol.u) == 51 and sol.stats["naccept"] == st["naccept"]
    err = np.max(np.abs(np.array(sol.u) - ref)) / 50.0
    assert err < 1e-10, err


@pytest.mark.parametrize("use_graph", [True, False])
def test_adaptive_readme_saveat(gpu_lib, use_graph):
    """README diffusion (test/README.jl): Tsit5 to t = 0.5 with saveat = 0.001.  use_graph runs
    the steps after the first accepted one as a device-side loop (conditional graph node)."""
    import fvmgpu as F

    spec = readme_diffusion(50)
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), saveat=0.001, use_graph=use_graph)
    assert len(sol.u) == 501 and np.isclose(sol.t[-1], 0.5)
    ref, st = _oracle_run(spec, list(sol.t))
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    err = np.max(np.abs(np.array(sol.u) - ref)) / 50.0
    assert err < 1e-8, err
    # sanity: the solution decays and stays within the initial bounds
    assert np.all(np.array(sol.u) <= 50 + 1e-9) and np.all(np.array(sol.u) >= -1e-9)


@pytest.mark.parametrize("use_graph", [True, False])
def test_adaptive_mixed_conditions(gpu_lib, use_graph):
    import fvmgpu as F

    spec = mixed_annulus()
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), saveat=0.02, use_graph=use_graph)
    ref, st = _oracle_run(spec, list(sol.t))
    err = np.max(np.abs(np.array(sol.u) - ref)) / np.max(np.abs(ref))
    assert err < 1e-8, err


def test_template_tsit5_matches_oracle(gpu_lib):
    import fvmgpu as F

    spec = sine_diffusion(40)
    mesh = F.FVMGeometry(spec.tri)
    BCs = F.BoundaryConditions(mesh, spec.bc_fns[0], F.Dirichlet)
    D = lambda x, y, p: spec.D(x, y, 0, 0, None)  # noqa: E731
    tmpl = F.DiffusionEquation(mesh, BCs, diffusion_function=D, initial_condition=spec.u0, final_time=1e-3)
    sol = F.solve(tmpl, F.Tsit5(), saveat=[1e-3], dt=5e-5, adaptive=False)
    assert sol.u[-1].shape[0] == spec.tri.num_points + 1 and sol.u[-1][-1] == 1.0
    conds = O.Conditions(spec.tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b, u0 = O.template_diffusion(spec.tri, conds, lambda x, y: D(x, y, None), spec.u0)
    ref, _ = O.tsit5_solve(lambda u, t: A @ u + b, u0, 0.0, 1e-3, [1e-3], dt=5e-5, adaptive=False)
    err = np.max(np.abs(sol.u[-1][:-1] - ref[-1])) / np.max(np.abs(ref[-1]))
    assert err < 1e-10, err


@pytest.mark.parametrize("side,driver", [(48, "cluster"), (96, "device_loop")])
def test_device_loop_matches_host_loop(gpu_lib, side, driver):
    """The device-side adaptive drivers (one thread-block cluster for the 2304-vertex mesh, the
    conditional-graph loop for the 9216-vertex one) and the host-controlled loop take the same
    steps: equal accept/reject counts and solutions equal to rounding, for saveat points that
    fall inside steps and on step ends (t0 and tf).  With a tiny given initial dt the first
    error estimates are rounding noise (the stages cancel to ~1e-16), so a last-bit difference
    between the device and host pow() (or the order of the error-norm sum) moves later step
    sizes: there the counts agree to within two steps and the solutions to the integration
    tolerance, 5e-4 of max|u| at reltol 1e-3 (the host loop itself is 1.7e-4 from the oracle
    there).  The cluster driver sums each row's products as a balanced
    tree (the other drivers sum them in slot order), so its solutions agree with the host loop
    to 1e-10 of max|u| rather than 1e-12."""
    import fvmgpu as F

    spec = sine_diffusion(side)
    spec.tf = 0.02
    prob = api_problem(spec)
    rt = 1e-10 if driver == "cluster" else 1e-12
    for kw, tol in (({"saveat": 0.0025}, rt), ({"saveat": [0.0, 0.013, 0.02]}, rt), ({"saveat": None}, rt),
                    ({"dt": 1e-5, "adaptive": True, "saveat": 0.005}, 5e-4)):
        a = F.solve(prob, F.Tsit5(), use_graph=True, **kw)
        b = F.solve(prob, F.Tsit5(), use_graph=False, **kw)
        assert a.stats["driver"] == driver and b.stats["driver"] == "host"
        if "dt" in kw:  # rounding-noise error estimates: the step sequences may part
            assert abs(a.stats["naccept"] - b.stats["naccept"]) <= 2 and abs(a.stats["nreject"] - b.stats["nreject"]) <= 2
        else:
            assert a.stats["naccept"] == b.stats["naccept"] and a.stats["nreject"] == b.stats["nreject"]
            assert a.stats["nrhs"] == b.stats["nrhs"]
        assert np.array_equal(np.asarray(a.t), np.asarray(b.t))
        ua, ub = np.array(a.u), np.array(b.u)
        assert np.max(np.abs(ua - ub)) <= tol * np.max(np.abs(ub)), kw


@pytest.mark.parametrize("side,use_graph", [(32, True), (96, True), (32, False)])
def test_adaptive_step_limit(gpu_lib, side, use_graph):
    """max_steps counts attempted steps; running out is an error on every driver (cluster,
    conditional-graph loop, host loop)."""
    import fvmgpu as F

    spec = sine_diffusion(side)
    spec.tf = 0.05
    prob = api_problem(spec)
    with pytest.raises(F.FVMError, match="max_steps"):
        F.solve(prob, F.Tsit5(), saveat=0.01, max_steps=5, use_graph=use_graph)


def test_cluster_wide_rows_and_dense_saves(gpu_lib):
    """The cluster driver on rows wider than 12 slots (a 40-spoke hub: the slot loop re-reads
    its slots instead of holding them in registers), a Robin boundary and a linear source,
    with 3001 saveat points (more than the 32 per step whose theta is shared):
    the same steps as the host loop, solutions equal to 1e-10 of max|u|."""
    import fvmgpu as F

    spec = wheel_diffusion(40)
    prob = api_problem(spec)
    ts = np.linspace(spec.t0, spec.tf, 3001)
    a = F.solve(prob, F.Tsit5(), saveat=ts, use_graph=True)
    b = F.solve(prob, F.Tsit5(), saveat=ts, use_graph=False)
    assert a.stats["driver"] == "cluster" and b.stats["driver"] == "host"
    assert a.stats["naccept"] == b.stats["naccept"] and a.stats["nreject"] == b.stats["nreject"]
    ua, ub = np.array(a.u), np.array(b.u)
    assert ua.shape == (3001, spec.tri.num_points)
    assert np.max(np.abs(ua - ub)) <= 1e-10 * np.max(np.abs(ub))


def test_device_loop_nonlinear_forms(gpu_lib):
    """Nonlinear forms (D(u), quadratic Neumann, logistic source) step through the
    conditional-graph loop with the per-triangle RHS inside the captured body: the same steps
    as the oracle's Tsit5, solutions within 1e-8 of max|u|."""
    import fvmgpu as F

    spec = nonlinear_rect(30)
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), saveat=0.002, use_graph=True)
    assert sol.stats["driver"] == "device_loop"
    ref, st = _oracle_run(spec, list(sol.t))
    assert sol.stats["naccept"] == st["naccept"] and sol.stats["nreject"] == st["nreject"]
    err = np.max(np.abs(np.array(sol.u) - ref)) / np.max(np.abs(ref))
    assert err < 1e-8, err
