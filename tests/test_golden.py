"""The committed README-problem fixture (tests/golden/c1_readme.npz, made by
tests/golden/make_golden.py from the oracle): the oracle still reproduces it (CPU), and the
GPU path matches it - RHS within 1e-12 of the term scale, the adaptive Tsit5 run with the
same accepted/rejected step counts and snapshots within 1e-8 of max|u| = 50."""
import os

import numpy as np
import pytest

import fvm_oracle as O
from problems import api_problem, oracle_problem, readme_diffusion, rhs_term_scale

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c1_readme.npz")


def _golden():
    return np.load(GOLDEN)


def test_oracle_reproduces_fixture():
    g = _golden()
    spec = readme_diffusion(50)
    prob = oracle_problem(spec)
    for u, du in ((g["u_rand"], g["du_rand"]), (spec.u0, g["du_u0"])):
        got = O.fvm_eqs(prob, u, 0.0)
        scale = np.linalg.norm(du) + np.linalg.norm(rhs_term_scale(prob, u, 0.0))
        assert np.linalg.norm(got - du) <= 1e-14 * scale


@pytest.mark.gpu
def test_gpu_matches_fixture(gpu_lib):
    import fvmgpu as F

    g = _golden()
    spec = readme_diffusion(50)
    oprob = oracle_problem(spec)
    prob = api_problem(spec)
    for u, du in ((g["u_rand"], g["du_rand"]), (spec.u0, g["du_u0"])):
        got = F.fvm_eqs(np.zeros_like(u), np.ascontiguousarray(u), prob, 0.0)
        scale = np.linalg.norm(du) + np.linalg.norm(rhs_term_scale(oprob, u, 0.0))
        assert np.linalg.norm(got - du) <= 1e-12 * scale
    sol = F.solve(prob, F.Tsit5(), saveat=list(g["t_save"]))
    assert sol.stats["naccept"] == int(g["naccept"]) and sol.stats["nreject"] == int(g["nreject"])
    assert np.max(np.abs(np.array(sol.u) - g["u_save"])) <= 1e-8 * 50.0


@pytest.mark.gpu
def test_gpu_matches_dense_saveat_fixture(gpu_lib):
    """The README's own run, saveat = 0.001 (501 saves, test/README.jl:4-15): the saves inside
    steps come from Tsit5's continuous extension on the GPU as in the oracle; 24 of them are
    frozen in the fixture.  Same step counts; within the adaptive-run tolerance, 1e-8 of
    max|u| = 50 (the step control's rounding differs in the last bits between the drivers)."""
    import fvmgpu as F

    g = _golden()
    spec = readme_diffusion(50)
    prob = api_problem(spec)
    sol = F.solve(prob, F.Tsit5(), saveat=0.001)
    assert len(sol.u) == 501
    assert sol.stats["naccept"] == int(g["naccept"]) and sol.stats["nreject"] == int(g["nreject"])
    got = np.array(sol.u)[g["k_dense"]]
    assert np.max(np.abs(got - g["u_dense"])) <= 1e-8 * 50.0


def test_oracle_reproduces_dense_saveat_fixture():
    g = _golden()
    spec = readme_diffusion(50)
    prob = oracle_problem(spec)
    cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
    snaps, _ = O.tsit5_solve(lambda u, t: O.fvm_eqs(prob, u, t), spec.u0, 0.0, 0.5, list(0.001 * g["k_dense"]),
                             callback=cb)
    assert np.max(np.abs(np.array(snaps) - g["u_dense"])) <= 1e-12 * 50.0


SYSTEM_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "system_gray_scott.npz")


def test_oracle_reproduces_system_fixture():
    """tests/golden/system_gray_scott.npz (the Gray-Scott tutorial FVMSystem on 30 x 30): the
    oracle's system restatement still gives the frozen RHS values and fixed-step solution."""
    from problems import gray_scott_oracle

    g = np.load(SYSTEM_GOLDEN)
    sys_ = gray_scott_oracle(30)
    for u, du in ((g["u_rand"], g["du_rand"]), (sys_.u0, g["du_u0"])):
        got = O.system_fvm_eqs(sys_, u, 0.0)
        # numpy's reductions may sum in another order on another build: a few ulps of the
        # largest value, not bit equality
        for c in range(2):
            assert np.max(np.abs(got[c] - du[c])) <= 1e-13 * np.max(np.abs(du[c]))
    snaps, _ = O.tsit5_solve(lambda u, t: O.system_fvm_eqs(sys_, u, t), sys_.u0, 0.0, 20.0, list(g["t_save"]),
                             dt=1.0, adaptive=False)
    # 20 steps, each a few ulps: relative to the solution's size
    assert np.max(np.abs(np.array(snaps) - g["u_save"])) <= 1e-13 * np.max(np.abs(g["u_save"]))


@pytest.mark.gpu
def test_gpu_matches_system_fixture(gpu_lib):
    import fvmgpu as F
    from test_gpu_system import gray_scott

    g = np.load(SYSTEM_GOLDEN)
    spec = gray_scott(30)
    spec.tf = 20.0  # the fixture's end time
    sys_ = spec.api()
    for u, du in ((g["u_rand"], g["du_rand"]), (spec.u0, g["du_u0"])):
        got = np.empty_like(u)
        sys_.rhs(got, np.ascontiguousarray(u), 0.0)
        for c in range(2):
            assert np.max(np.abs(got[c] - du[c])) <= 1e-12 * np.max(np.abs(du[c]))
    sol = F.solve(sys_, F.Tsit5(), saveat=list(g["t_save"]), dt=1.0, adaptive=False)
    assert np.max(np.abs(np.array(sol.u) - g["u_save"])) <= 1e-11
