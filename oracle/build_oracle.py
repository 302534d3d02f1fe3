"""Build recipe of the oracle's C restatement (TEST / BASELINE INFRASTRUCTURE).

Compiles oracle/fvm_oracle_c.c into oracle/build/liborc.so with gcc -O3 -fopenmp, and wraps
it with ctypes for the tests and bench.py's CPU-baseline leg.  The reference itself is pure
Julia (no C/C++ sources), so there is nothing of the reference to compile here.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "fvm_oracle_c.c"
LIB = HERE / "build" / "liborc.so"

D_CONST, D_SINE, D_JUMP = 0, 1, 2


class OrcProblem(C.Structure):
    _fields_ = [
        ("np", C.c_int64), ("nt", C.c_int64), ("nbe", C.c_int64),
        ("tri", C.POINTER(C.c_int32)), ("props", C.POINTER(C.c_double)), ("pts", C.POINTER(C.c_double)),
        ("vol", C.POINTER(C.c_double)), ("bedge", C.POINTER(C.c_int32)), ("code", C.POINTER(C.c_int8)),
        ("d_kind", C.c_int), ("d_param", C.c_double * 4),
    ]


class GrayScott(C.Structure):
    _fields_ = [("eps", C.c_double * 2), ("b", C.c_double), ("d", C.c_double)]


def build(force: bool = False) -> Path:
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", str(SRC), "-o", str(LIB) + ".tmp",
               "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"oracle build failed: {r.stderr}")
        Path(str(LIB) + ".tmp").replace(LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.orc_rhs_serial.argtypes = [C.POINTER(OrcProblem), C.c_void_p, C.c_void_p, C.c_double]
        lib.orc_rhs_threaded.argtypes = [C.POINTER(OrcProblem), C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                         C.c_void_p]
        lib.orc_max_threads.restype = C.c_int
        lib.orc_steady_bicgstab.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_double, C.c_void_p, C.c_double, C.c_int64, C.c_double, C.c_int,
                                            C.c_void_p, C.c_void_p]
        lib.orc_gray_scott_rhs_threaded.argtypes = [C.POINTER(OrcProblem), C.POINTER(GrayScott), C.c_void_p,
                                                    C.c_void_p, C.c_int, C.c_void_p]
        _lib = lib
    return _lib


class CProblem:
    """The C restatement's problem for a diffusion FVMProblem with a built-in D closure and
    Dirichlet / free vertex codes (the benchmark configurations)."""

    def __init__(self, geo, tri, code, d_kind, d_param, bnd_tri):
        self.keep = [np.ascontiguousarray(tri.triangles, dtype=np.int32),
                     np.ascontiguousarray(np.concatenate([geo.s, geo.mid.reshape(-1, 6), geo.nrm.reshape(-1, 6),
                                                          geo.length], axis=1)),
                     np.ascontiguousarray(tri.points, dtype=np.float64),
                     np.ascontiguousarray(geo.cv_volumes),
                     np.ascontiguousarray(np.concatenate([tri.boundary_edges, bnd_tri.reshape(-1, 1)], axis=1),
                                          dtype=np.int32),
                     np.ascontiguousarray(code, dtype=np.int8)]
        p = OrcProblem()
        p.np, p.nt, p.nbe = tri.num_points, tri.num_triangles, tri.num_boundary_edges
        p.tri = self.keep[0].ctypes.data_as(C.POINTER(C.c_int32))
        p.props = self.keep[1].ctypes.data_as(C.POINTER(C.c_double))
        p.pts = self.keep[2].ctypes.data_as(C.POINTER(C.c_double))
        p.vol = self.keep[3].ctypes.data_as(C.POINTER(C.c_double))
        p.bedge = self.keep[4].ctypes.data_as(C.POINTER(C.c_int32))
        p.code = self.keep[5].ctypes.data_as(C.POINTER(C.c_int8))
        p.d_kind = d_kind
        for i, v in enumerate(d_param[:4]):
            p.d_param[i] = v
        self.p = p
        self.np = tri.num_points
        self._dup = None

    def rhs_serial(self, u, t=0.0):
        du = np.empty(self.np)
        load().orc_rhs_serial(C.byref(self.p), u.ctypes.data, du.ctypes.data, t)
        return du

    def rhs_threaded(self, u, t=0.0, nthreads=0, du=None):
        lib = load()
        nth = nthreads or lib.orc_max_threads()
        if self._dup is None or self._dup.size < self.np * nth:
            self._dup = np.empty(self.np * nth)
        du = np.empty(self.np) if du is None else du
        lib.orc_rhs_threaded(C.byref(self.p), u.ctypes.data, du.ctypes.data, t, nth, self._dup.ctypes.data)
        return du


class CGrayScott(CProblem):
    """The C restatement of the Gray-Scott tutorial FVMSystem (zero Neumann boundary, fluxes
    -eps_c grad u_c, sources b (1 - u) - u v^2 and -d v + u v^2); state (2, npoints) as the
    reference's matrix, passed in its [point][component] memory order."""

    def __init__(self, geo, tri, code, bnd_tri, eps=(2e-5, 1e-5), b=0.04, d=0.1):
        super().__init__(geo, tri, code, D_CONST, (0.0,), bnd_tri)
        self.g = GrayScott()
        self.g.eps[0], self.g.eps[1] = eps
        self.g.b, self.g.d = b, d

    def rhs_threaded(self, u, t=0.0, nthreads=0, du=None):
        """u, du: (2, npoints) arrays; du is returned."""
        lib = load()
        nth = nthreads or lib.orc_max_threads()
        if self._dup is None or self._dup.size < 2 * self.np * nth:
            self._dup = np.empty(2 * self.np * nth)
        ut = np.ascontiguousarray(np.asarray(u, dtype=np.float64).T)
        dt = np.empty_like(ut)
        lib.orc_gray_scott_rhs_threaded(C.byref(self.p), C.byref(self.g), ut.ctypes.data, dt.ctypes.data, nth,
                                        self._dup.ctypes.data)
        if du is None:
            return dt.T.copy()
        du[...] = dt.T
        return du


def reduced_system(A, b, V):
    """The steady template's system A x = b as the GPU solver takes it: rows fixed by a
    Dirichlet condition or a missing vertex (identity rows of A) stay identity rows with a zero
    right-hand side, their columns move into the right-hand side of the free rows, and free rows
    are scaled by -V.  Returns (B, rhs, xfix, w) with x = z + xfix for B z = rhs, and
    (b - A x)_i = -(rhs - B z)_i / V_i on free rows (w = 1 / V there, 0 on fixed rows)."""
    from scipy.sparse import csr_matrix, diags

    A = A.tocsr()
    n = A.shape[0]
    nnz_row = np.diff(A.indptr)
    fixed = (nnz_row == 1) & np.isclose(A.diagonal(), 1.0) & (np.asarray(abs(A).sum(axis=1)).ravel() == 1.0)
    xfix = np.where(fixed, b, 0.0)
    M = A.tocoo()
    keep = ~fixed[M.row] & ~fixed[M.col]
    Bf = csr_matrix((M.data[keep], (M.row[keep], M.col[keep])), shape=A.shape)
    rhs_free = b - A @ xfix
    sc = np.where(fixed, 1.0, -V)
    B = (diags(sc) @ Bf).tocsr() + diags(np.where(fixed, 1.0, 0.0))
    rhs = np.where(fixed, 0.0, sc * rhs_free)
    w = np.where(fixed, 0.0, 1.0 / np.where(fixed, 1.0, V))
    return B.tocsr(), rhs, xfix, w


def steady_bicgstab(A, b, rtol=1e-10, maxit=200_000, nthreads=0, max_seconds=1e9, V=None):
    """Jacobi-preconditioned FP64 BiCGStab on the host threads (the CPU baseline of the steady
    templates), stopped at ||b - A x|| / ||b|| <= rtol, maxit or max_seconds.  With the control
    volumes V it solves the GPU solver's reduced system (reduced_system) instead of A x = b
    directly.  Returns (x, {"iterations", "rel_residual", "converged", "seconds", "threads"})."""
    import time

    lib = load()
    A = A.tocsr()
    n = A.shape[0]
    bnorm = float(np.linalg.norm(b))
    if V is not None:
        M, rhs, xfix, w = reduced_system(A, b, V)
    else:
        M, rhs, xfix, w = A, np.asarray(b, dtype=np.float64), np.zeros(n), None
    rp = np.ascontiguousarray(M.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(M.indices, dtype=np.int32)
    va = np.ascontiguousarray(M.data, dtype=np.float64)
    bb = np.ascontiguousarray(rhs, dtype=np.float64)
    wp = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    z = np.zeros(n)
    work = np.empty(8 * n)
    st = np.zeros(3)
    nth = nthreads or lib.orc_max_threads()
    t0 = time.perf_counter()
    lib.orc_steady_bicgstab(n, rp.ctypes.data, ci.ctypes.data, va.ctypes.data, bb.ctypes.data,
                            None if wp is None else wp.ctypes.data, bnorm, z.ctypes.data, float(rtol), int(maxit),
                            float(max_seconds), int(nth), work.ctypes.data, st.ctypes.data)
    dt = time.perf_counter() - t0
    return z + xfix, {"iterations": int(st[0]), "rel_residual": float(st[1]), "converged": bool(st[2]),
                      "seconds": dt, "threads": nth}


def max_threads() -> int:
    return load().orc_max_threads()
