"""The C restatement used as the timed CPU baseline agrees with the numpy oracle
(serial and threaded, the latter mirroring parallel_fvm_eqs!)."""
import numpy as np

import build_oracle as B
import fvm_oracle as O
from problems import oracle_problem, readme_diffusion, sine_diffusion


def _cproblem(spec, kind, param):
    prob = oracle_problem(spec)
    return prob, B.CProblem(prob.geo, spec.tri, prob.code, kind, param, prob.bnd_tri)


def test_c_oracle_matches_numpy_oracle():
    for spec, kind, param in ((readme_diffusion(50), B.D_CONST, (1 / 9,)), (sine_diffusion(40), B.D_SINE, (0.5,))):
        prob, cp = _cproblem(spec, kind, param)
        u = spec.u0 + np.random.default_rng(0).random(spec.tri.num_points)
        ref = O.fvm_eqs(prob, u, 0.0)
        for got in (cp.rhs_serial(u), cp.rhs_threaded(u, nthreads=3), cp.rhs_threaded(u, nthreads=1)):
            assert np.linalg.norm(got - ref) <= 1e-13 * np.linalg.norm(ref)
