"""Generates tests/golden/c1_readme.npz (and system_gray_scott.npz, see compute_system): frozen
oracle outputs for the README diffusion problem
(test/README.jl:4-15 of the reference: triangulate_rectangle(0, 2, 0, 2, 50, 50,
single_boundary=true), zero Dirichlet, D = 1/9, u0 = 50 where y <= 1 else 0).

Arrays (caller numbering, 2500 points):
  u_rand, du_rand   a seeded random field (seed 20) and fvm_eqs! of it at t = 0
  du_u0             fvm_eqs! of the initial condition
  t_save, u_save    adaptive Tsit5 (abstol 1e-6, reltol 1e-3, the Dirichlet callback after
                    every step) at t = 0.01, 0.1, 0.25, 0.5
  naccept, nreject  the step counts of that run
  k_dense, u_dense  24 of the 501 saves of the README's saveat = 0.001 run (t = 0.001 k_dense;
                    the steps do not depend on saveat, so any subset of the grid gives the same
                    values), interpolated inside the steps by Tsit5's continuous extension

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
from problems import gray_scott_oracle, oracle_problem, readme_diffusion  # noqa: E402

T_SAVE = [0.01, 0.1, 0.25, 0.5]


def compute():
    spec = readme_diffusion(50)
    prob = oracle_problem(spec)
    u_rand = 50.0 * np.random.default_rng(20).random(spec.tri.num_points)
    du_rand = O.fvm_eqs(prob, u_rand, 0.0)
    du_u0 = O.fvm_eqs(prob, spec.u0, 0.0)
    cb = lambda u, t: O.update_dirichlet_nodes(prob, u, t)  # noqa: E731
    snaps, st = O.tsit5_solve(lambda u, t: O.fvm_eqs(prob, u, t), spec.u0, 0.0, 0.5, T_SAVE, callback=cb)
    k_dense = np.sort(np.random.default_rng(22).choice(501, size=24, replace=False))
    dense, st2 = O.tsit5_solve(lambda u, t: O.fvm_eqs(prob, u, t), spec.u0, 0.0, 0.5, list(0.001 * k_dense),
                               callback=cb)
    assert st2["naccept"] == st["naccept"] and st2["nreject"] == st["nreject"]
    return {"u_rand": u_rand, "du_rand": du_rand, "du_u0": du_u0, "t_save": np.array(T_SAVE),
            "u_save": np.array(snaps), "naccept": np.array(st["naccept"]), "nreject": np.array(st["nreject"]),
            "k_dense": k_dense, "u_dense": np.array(dense)}


def compute_system():
    """tests/golden/system_gray_scott.npz: the Gray-Scott tutorial FVMSystem (tests/problems.py:
    gray_scott_oracle) on 30 x 30.  u_rand (seed 21) and system fvm_eqs! of it; du_u0 of the
    initial condition; u_save at t_save from fixed-step Tsit5 (dt = 1) started at u0."""
    sys_ = gray_scott_oracle(30)
    u_rand = np.random.default_rng(21).random(sys_.u0.shape)
    t_save = np.array([0.0, 5.0, 20.0])
    snaps, _ = O.tsit5_solve(lambda u, t: O.system_fvm_eqs(sys_, u, t), sys_.u0, 0.0, 20.0, list(t_save), dt=1.0,
                             adaptive=False)
    return {"u_rand": u_rand, "du_rand": O.system_fvm_eqs(sys_, u_rand, 0.0),
            "du_u0": O.system_fvm_eqs(sys_, sys_.u0, 0.0), "t_save": t_save, "u_save": np.array(snaps)}


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "c1_readme.npz"), **compute())
    np.savez_compressed(os.path.join(here, "system_gray_scott.npz"), **compute_system())
