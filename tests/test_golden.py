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
