"""Generates tests/golden/c1_readme.npz: frozen oracle outputs for the README diffusion problem
(test/README.jl:4-15 of the reference: triangulate_rectangle(0, 2, 0, 2, 50, 50,
single_boundary=true), zero Dirichlet, D = 1/9, u0 = 50 where y <= 1 else 0).

Arrays (caller numbering, 2500 points):
  u_rand, du_rand   a seeded random field (seed 20) and fvm_eqs! of it at t = 0
  du_u0             fvm_eqs! of the initial condition
  t_save, u_save    adaptive Tsit5 (abstol 1e-6, reltol 1e-3, the Dirichlet callback after
                    every step) at t = 0.01, 0.1, 0.25, 0.5
  naccept, nreject  the step counts of that run

The reference itself cannot run here (pure Julia, no Julia on any machine), so the fixture
freezes the oracle, which is pinned by the reference's known-answer tests; it guards the
oracle against drift and gives the GPU tests a fixed target.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"),
                os.path.join(ROOT, "finitevolumemethod.jl_gb300")]

import fvm_oracle as O  # noqa: E402
from problems import oracle_problem, readme_diffusion  # noqa: E402

T_SAVE = [0.01, 0.1, 0.25, 0.5]


def compute():
    spec = readme_diffusion(50)
    prob = oracle_problem(spec)
    u_rand = 50.0 * np.random.default_rng(20).random(spec.tri.num_points)
    du_rand = O.fvm_eqs(prob, u_rand, 0.0)
    du_u0 = O.fvm_eqs(prob, spec.u0, 0.0)
    cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
    snaps, st = O.tsit5_solve(lambda u, t: O.fvm_eqs(prob, u, t), spec.u0, 0.0, 0.5, T_SAVE, callback=cb)
    return {"u_rand": u_rand, "du_rand": du_rand, "du_u0": du_u0, "t_save": np.array(T_SAVE),
            "u_save": np.array(snaps), "naccept": np.array(st["naccept"]), "nreject": np.array(st["nreject"])}


if __name__ == "__main__":
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "c1_readme.npz"), **compute())
