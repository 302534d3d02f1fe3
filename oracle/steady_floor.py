"""Residual floor of an FP64 solution of the disk Poisson system (MEASUREMENT INFRASTRUCTURE).

For the oracle's PoissonsEquation assembly on the disk workload (triangulate_disk(N, 4096,
seed=0), D = 1 for r < 0.5 and 10 otherwise, f = -1, zero Dirichlet; the reference's
poissons_equation.jl:58-88), solves A x = b by sparse LU with two refinement steps whose
residuals are formed in extended precision (numpy longdouble), rounds x to FP64 and prints
||b - A fl(x)|| / ||b|| evaluated in extended precision.  No FP64 vector can be expected to do
much better, so this bounds the relative residual any FP64 steady solve reaches.  Measured:
7.52e-11 at N = 500,000 and 4.03e-10 at N = 2,000,000 (the FP64-evaluated residual of the same
vector is 9.0e-11 and 8.3e-10).

    python oracle/steady_floor.py 500000
"""
import sys
import time
from pathlib import Path

import numpy as np
import scipy.sparse.linalg as sla

ROOT = Path(__file__).resolve().parent.parent
for _p in (ROOT / "finitevolumemethod.jl_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import fvm_oracle as O  # noqa: E402
from fvmgpu.meshes import triangulate_disk  # noqa: E402


def floor(npts, seed=0):
    tri = triangulate_disk(npts, 4096, seed=seed)
    conds = O.Conditions(tri, [lambda x, y, t, u: 0.0 * x], ["Dirichlet"])
    A, b = O.template_poisson(tri, conds, lambda x, y: np.where(x * x + y * y < 0.25, 1.0, 10.0),
                              lambda x, y: -1.0 + 0.0 * x)
    A = A.tocsr()
    Al = A.astype(np.longdouble)
    bl = b.astype(np.longdouble)
    lu = sla.splu(A.tocsc())
    x = lu.solve(b).astype(np.longdouble)
    for _ in range(2):
        r = bl - Al @ x
        x = x + lu.solve(r.astype(np.float64)).astype(np.longdouble)
    xr = x.astype(np.float64)
    r = bl - Al @ xr.astype(np.longdouble)
    exact = float(np.sqrt(np.sum(r * r)) / np.sqrt(np.sum(bl * bl)))
    fp64 = float(np.linalg.norm(b - A @ xr) / np.linalg.norm(b))
    return exact, fp64


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 500_000
    t0 = time.time()
    e, f = floor(n)
    print(f"N={n}: ||b - A fl(x*)|| / ||b|| = {e:.3e} (extended precision), {f:.3e} (FP64 evaluation); "
          f"{time.time() - t0:.0f} s")
