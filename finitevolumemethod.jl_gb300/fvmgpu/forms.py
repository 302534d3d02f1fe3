"""Closures -> device-coded forms.

Julia (and Python) closures are opaque to the GPU.  The host evaluates each closure at the
points where the reference would evaluate it (vertices, dual-edge midpoints, boundary
quarter points) and classifies it:

* a closure of (x, y) alone is sampled into a per-point array;
* a closure that is a polynomial of degree <= 2 in u with (x, y)-dependent coefficients
  becomes the coefficient arrays c0, c1, c2 (f = c0 + c1 u + c2 u^2);
* where the caller allows it (conditions and sources of linear problems), the constant term
  c0 may depend on t through one factor of a fixed set: c0(x, y, t) = A(x, y) + tau(t) B(x, y)
  with tau(t) = exp(a (t - t0)) or 1 + a (t - t0) + b (t - t0)^2 (`TimeFactor`);
* anything else (other t dependence, non-polynomial u dependence, non-finite values) is
  rejected with `UnsupportedFormError`: never guessed.

Classification probes the closure at u in {0, 1, -1} and t in {t0, t0 + 1.37}, fits the
quadratic, and verifies it at u in {2, -0.5, 3.25} and at the second time, to a relative
tolerance of 1e-10 (two verifications at every point, the rest on a subsample).  A time factor is fitted from c0 at six equally spaced times across
[t0, tf] and verified at three other times, to the same tolerance.
"""
from __future__ import annotations

import numpy as np

from ._lib import UnsupportedFormError, FVM_ERR_UNSUPPORTED_FORM

_FIT_U = (0.0, 1.0, -1.0)
_CHECK_U = (2.0, -0.5, 3.25)
_RTOL = 1e-10


def evaluate(f, *args):
    """Call f at broadcast numpy arguments (None passes through); per-point fallback when the
    closure does not accept arrays (e.g. it branches on a coordinate)."""
    arrs = [None if a is None else np.asarray(a, dtype=np.float64) for a in args]
    shapes = [a.shape for a in arrs if a is not None]
    shape = np.broadcast_shapes(*shapes) if shapes else ()
    try:
        with np.errstate(all="ignore"):
            out = f(*arrs)
        if isinstance(out, tuple):
            return tuple(np.broadcast_to(np.asarray(o, dtype=np.float64), shape).copy() for o in out)
        return np.broadcast_to(np.asarray(out, dtype=np.float64), shape).copy()
    except (ValueError, TypeError):
        pass
    flat = [None if a is None else np.broadcast_to(a, shape).ravel() for a in arrs]
    n = int(np.prod(shape)) if shape else 1
    res = None
    for m in range(n):
        r = f(*[None if a is None else float(a[m]) for a in flat])
        if res is None:
            res = [np.empty(n) for _ in r] if isinstance(r, tuple) else np.empty(n)
        if isinstance(r, tuple):
            for c, v in enumerate(r):
                res[c][m] = v
        else:
            res[m] = r
    if isinstance(res, list):
        return tuple(r.reshape(shape) for r in res)
    return res.reshape(shape)


def _reject(what, why):
    raise UnsupportedFormError(FVM_ERR_UNSUPPORTED_FORM, f"{what}: {why}; supported forms are closures of (x, y) "
                               "and polynomials of degree <= 2 in u with (x, y) coefficients, independent of t "
                               "except for a constant term A(x, y) + tau(t) B(x, y), tau(t) = exp(a (t - t0)) or "
                               "1 + a (t - t0) + b (t - t0)^2, in the conditions and source of a linear problem")


class TimeFactor(tuple):
    """(kind, t_ref, a, b): kind 1 is tau(t) = exp(a (t - t_ref)), kind 2 is
    tau(t) = 1 + a (t - t_ref) + b (t - t_ref)^2 (the descriptor's time_factor rows)."""

    def __new__(cls, kind, t_ref, a, b=0.0):
        return super().__new__(cls, (float(kind), float(t_ref), float(a), float(b)))

    def __call__(self, t):
        d = np.asarray(t, dtype=np.float64) - self[1]
        return np.exp(self[2] * d) if self[0] == 1.0 else 1.0 + d * (self[2] + d * self[3])

    def close_to(self, other, rtol=1e-11):
        return (self[0] == other[0] and self[1] == other[1]
                and all(abs(p - q) <= rtol * max(abs(p), abs(q), 1e-300) for p, q in zip(self[2:], other[2:])))


def fit_time_factor(c0_at, t0, tf, what):
    """Fit c0(t) = A + tau(t) B (arrays over points) for tau in the device set, from c0 at six
    equally spaced times across [t0, tf]; verify at three other times.  Returns
    (A, TimeFactor, B), or None when c0 does not depend on t.  Rejects other t dependence."""
    t0 = float(t0)
    span = float(tf) - t0 if tf is not None and np.isfinite(float(tf)) and float(tf) > t0 else 1.0
    h = span / 5
    C = [np.asarray(c0_at(t0 + k * h), dtype=np.float64) for k in range(6)]
    scale = max(float(np.max(np.abs(c))) if c.size else 0.0 for c in C)
    tol = _RTOL * max(scale, 1e-300)
    for c in C:
        if not np.all(np.isfinite(c)):
            _reject(what, "non-finite values")
    D = [c - C[0] for c in C]
    if all(np.all(np.abs(d) <= tol) for d in D):
        return None
    w = max(D[1:], key=lambda d: float(np.max(np.abs(d))))
    ww = float(np.dot(w, w))
    s = np.array([float(np.dot(d, w)) / ww for d in D])  # D_k = s_k w
    if not all(np.all(np.abs(d - sk * w) <= tol) for d, sk in zip(D, s)):
        _reject(what, "depends on t other than through one factor tau(t)")
    smax = float(np.max(np.abs(s)))
    fits = []
    # exponential: differences of s form a geometric sequence with ratio exp(a h)
    if abs(s[1]) > 1e-8 * smax:
        rho = (s[2] - s[1]) / s[1]
        if rho > 0 and abs(rho - 1) > 1e-6:
            a = np.log(rho) / h
            cexp = s[1] / (rho - 1)
            pred = cexp * (np.exp(a * h * np.arange(6)) - 1)
            if np.all(np.abs(pred - s) <= 1e-10 * smax):
                fits.append((TimeFactor(1, t0, a), cexp))
    if not fits:  # polynomial: s_k = alpha k + beta k^2
        k = np.arange(6, dtype=np.float64)
        M = np.stack([k, k * k], axis=1)
        (al, be), *_ = np.linalg.lstsq(M, s, rcond=None)
        # a coefficient at the rounding level of the other is zero (so equal factors compare equal)
        if abs(be) <= 1e-12 * abs(al):
            be = 0.0
        elif abs(al) <= 1e-12 * abs(be):
            al = 0.0
        if np.all(np.abs(M @ np.array([al, be]) - s) <= 1e-10 * smax):
            fits.append((TimeFactor(2, t0, al / h, be / (h * h)), 1.0))
    if not fits:
        _reject(what, "depends on t other than through exp(a (t - t0)) or a quadratic in t - t0")
    tau, cs = fits[0]
    B = cs * w
    A = C[0] - B
    for frac in (0.31, 2.77, 4.43):
        t = t0 + frac * h
        if not np.all(np.abs(np.asarray(c0_at(t)) - (A + tau(t) * B)) <= tol):
            _reject(what, "depends on t other than through exp(a (t - t0)) or a quadratic in t - t0")
    return A, tau, B


def classify_xytu(f, x, y, t0, what, max_degree=2, tf=None, time=False):
    """Coefficients (c0, c1, c2)[:deg+1] and degree of g(x, y, t, u) = f(x, y, t, u) at points.

    The closure is evaluated at every point five times: the fit at u = 0, 1, -1, and two
    verifications, u = 2 at t0 and u = -0.5 at the second time, which catch a part that is not
    quadratic in u, or that depends on t, at any point.  The other probes (u = -0.5 and 3.25 at
    t0, the fit values at the second time) run on a subsample of about 4096 points.

    time=True allows c0 to depend on t through one factor (`fit_time_factor` over [t0, tf]);
    then returns (coeffs, deg, tpart) with coeffs[..., 0] the static part A and tpart
    (TimeFactor, B) or None."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = x.shape[0] if x.ndim else 1
    t1 = float(t0)
    t2 = t1 + 1.37
    sub = slice(None, None, max(1, n // 4096)) if x.ndim else slice(None)

    def ev(t, u, at=slice(None)):
        xs, ys = (x[at], y[at]) if x.ndim else (x, y)
        try:
            return evaluate(f, xs, ys, t, np.full(xs.shape, u))
        except Exception as e:  # noqa: BLE001
            _reject(what, f"evaluation failed ({e!r})")

    g = {u: ev(t1, u) for u in _FIT_U}
    for v in g.values():
        if not np.all(np.isfinite(v)):
            _reject(what, "non-finite values")
    c0 = g[0.0]
    c1 = (g[1.0] - g[-1.0]) / 2
    c2 = (g[1.0] + g[-1.0]) / 2 - c0
    scale = np.maximum(np.maximum(np.abs(c0), np.abs(c1)), np.abs(c2))
    scale = np.maximum(scale, np.max(scale) * 1e-300 + 1e-300)
    B = np.zeros_like(c0)
    tau = None

    def fit_time(at):
        return fit_time_factor(lambda t: ev(t, 0.0, at), t1, tf, what)

    if time and fit_time(sub) is not None:  # the factor, fitted at every point
        _, tau, B = fit_time(slice(None))

    def check(t, u, at, why):
        got = ev(t, u, at)
        dt = 0.0 if tau is None else tau(t) - 1.0
        pred = c0[at] + dt * B[at] + u * (c1[at] + u * c2[at])
        sc = np.maximum(scale[at], np.abs(dt * B[at]))
        if not np.all(np.abs(got - pred) <= _RTOL * (sc * (1 + abs(u)) ** 2)):
            _reject(what, why)

    poly = "not a polynomial of degree <= 2 in u"
    tdep = "depends on t" + (" in its u-dependent terms" if time else "")
    check(t1, 2.0, slice(None), poly)
    if time and tau is None:
        # a t dependence the subsample missed: fit it at every point before the full check
        try:
            check(t2, -0.5, slice(None), tdep)
        except UnsupportedFormError:
            fit = fit_time(slice(None))
            if fit is None:
                raise
            _, tau, B = fit
    check(t2, -0.5, slice(None), tdep)
    for u in _CHECK_U[1:]:
        check(t1, u, sub, poly)
    for u in _FIT_U:
        check(t2, u, sub, tdep)
    if tau is not None:
        c0 = c0 - B
    tiny = 1e-14 * np.max(scale) if scale.size else 0.0
    if np.all(np.abs(c2) <= tiny):
        c2 = np.zeros_like(c2)
        if np.all(np.abs(c1) <= tiny):
            c1 = np.zeros_like(c1)
    deg = 2 if np.any(c2 != 0) else (1 if np.any(c1 != 0) else 0)
    if deg > max_degree:
        _reject(what, f"degree {deg} in u exceeds {max_degree}")
    coeffs = np.stack([c0, c1, c2][: deg + 1], axis=-1)
    if time:
        return coeffs, deg, (None if tau is None else (tau, B))
    return coeffs, deg


def classify_flux(q, x, y, t0, what="flux_function"):
    """D(x, y) of a flux q(x, y, t, alpha, beta, gamma) = -D(x, y) (alpha, beta), or reject.

    Probes (alpha, beta, gamma) = (1,0,0), (0,1,0), (0,0,1) and verifies linearity at
    (2, -3, 5) and at a second time."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    ones = np.ones(x.shape)
    zero = np.zeros(x.shape)

    def ev(a, b, c, t=t0):
        try:
            qx, qy = evaluate(q, x, y, t, a * ones, b * ones, c * ones)
        except Exception as e:  # noqa: BLE001
            _reject(what, f"evaluation failed ({e!r})")
        return qx, qy

    ax, ay = ev(1.0, 0.0, 0.0)
    bx, by = ev(0.0, 1.0, 0.0)
    gx, gy = ev(0.0, 0.0, 1.0)
    zx, zy = ev(0.0, 0.0, 0.0)
    D = -ax
    scale = np.maximum(np.abs(D), 1e-300)
    ok = (np.all(np.abs(ay) <= _RTOL * scale) and np.all(np.abs(bx) <= _RTOL * scale)
          and np.all(np.abs(by + D) <= _RTOL * scale) and np.all(np.abs(gx) <= _RTOL * scale)
          and np.all(np.abs(gy) <= _RTOL * scale) and np.all(np.abs(zx) <= _RTOL * scale)
          and np.all(np.abs(zy) <= _RTOL * scale))
    if ok:
        cx, cy = ev(2.0, -3.0, 5.0, t0 + 1.37)
        ok = np.all(np.abs(cx + 2 * D) <= _RTOL * 4 * scale) and np.all(np.abs(cy - 3 * D) <= _RTOL * 4 * scale)
    if not ok or not np.all(np.isfinite(D)):
        _reject(what, "not of the form -D(x, y) (alpha, beta)")
    return D


def classify_linear_flux(q, x, y, t0, what="flux_function"):
    """M (npoints, 6) of a flux linear in (alpha, beta, gamma),
    q(x, y, t, alpha, beta, gamma) = (M0 alpha + M1 beta + M2 gamma, M3 alpha + M4 beta + M5 gamma),
    with M depending on (x, y) only (e.g. the advection-diffusion flux nu u - D grad u with
    u = alpha x + beta y + gamma), or reject.  Probes the unit vectors and zero, and verifies
    linearity at (2, -3, 5) and at a second time, relative to the size of the summed terms."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    ones = np.ones(x.shape)

    def ev(a, b, c, t=t0):
        try:
            qx, qy = evaluate(q, x, y, t, a * ones, b * ones, c * ones)
        except Exception as e:  # noqa: BLE001
            _reject(what, f"evaluation failed ({e!r})")
        return np.asarray(qx, dtype=np.float64) * ones, np.asarray(qy, dtype=np.float64) * ones

    zx, zy = ev(0.0, 0.0, 0.0)
    cols = [ev(1.0, 0.0, 0.0), ev(0.0, 1.0, 0.0), ev(0.0, 0.0, 1.0)]
    M = np.stack([cols[0][0] - zx, cols[1][0] - zx, cols[2][0] - zx,
                  cols[0][1] - zy, cols[1][1] - zy, cols[2][1] - zy], axis=1)
    if not np.all(np.isfinite(M)):
        _reject(what, "non-finite values")
    big = np.max(np.abs(M), axis=1)
    ok = np.all(np.abs(zx) <= _RTOL * big) and np.all(np.abs(zy) <= _RTOL * big)
    if ok:
        a, b, c = 2.0, -3.0, 5.0
        cx, cy = ev(a, b, c, t0 + 1.37)
        px = M[:, 0] * a + M[:, 1] * b + M[:, 2] * c
        py = M[:, 3] * a + M[:, 4] * b + M[:, 5] * c
        tx = np.abs(M[:, 0] * a) + np.abs(M[:, 1] * b) + np.abs(M[:, 2] * c)
        ty = np.abs(M[:, 3] * a) + np.abs(M[:, 4] * b) + np.abs(M[:, 5] * c)
        ok = np.all(np.abs(cx - px) <= _RTOL * tx + 1e-300) and np.all(np.abs(cy - py) <= _RTOL * ty + 1e-300)
    if not ok:
        _reject(what, "not linear in (alpha, beta, gamma) with coefficients of (x, y)")
    return np.ascontiguousarray(M)


def sample_xy(f, x, y, *extra, what="function"):
    """Values of a closure of (x, y[, extra...]) at points (template closures, ICs)."""
    try:
        v = evaluate(f, x, y, *extra)
    except Exception as e:  # noqa: BLE001
        _reject(what, f"evaluation failed ({e!r})")
    if not np.all(np.isfinite(v)):
        _reject(what, "non-finite values")
    return v


# --------------------------------------------------------------------------------------
# systems (FVMSystem): closures take N-tuples -- alpha, beta, gamma for fluxes, the node's
# component values u = (u_1, ..., u_N) for sources and conditions
# --------------------------------------------------------------------------------------
_SYS_DEGREE = 3


def evaluate_tuples(f, x, y, t, *tuples):
    """Call f(x, y, t, T1, T2, ...) whose Ti are N-tuples of values (scalars, the same at every
    point, or arrays over the points).  Scalars are passed as scalars first, so work that does
    not depend on the point is done once; a closure that needs arrays gets them broadcast; one
    that takes neither is called once per point with tuples of floats."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    y = np.broadcast_to(np.asarray(y, dtype=np.float64), (n,))
    T = [tuple(np.broadcast_to(np.asarray(c, dtype=np.float64), (n,)) for c in tup) for tup in tuples]
    attempts = []
    if any(np.ndim(c) == 0 for tup in tuples for c in tup):
        attempts.append([tuple(np.float64(c) if np.ndim(c) == 0 else Tc for c, Tc in zip(tup, Ttup))
                         for tup, Ttup in zip(tuples, T)])
    attempts.append(T)
    for args in attempts:
        try:
            with np.errstate(all="ignore"):
                out = f(x, y, t, *args)
            if isinstance(out, tuple):
                return tuple(np.broadcast_to(np.asarray(o, dtype=np.float64), (n,)).copy() for o in out)
            return np.broadcast_to(np.asarray(out, dtype=np.float64), (n,)).copy()
        except (ValueError, TypeError, IndexError):
            pass
    res = None
    for m in range(n):
        r = f(float(x[m]), float(y[m]), t, *[tuple(float(c[m]) for c in tup) for tup in T])
        if res is None:
            res = [np.empty(n) for _ in r] if isinstance(r, tuple) else np.empty(n)
        if isinstance(r, tuple):
            for c, v in enumerate(r):
                res[c][m] = v
        else:
            res[m] = r
    return tuple(res) if isinstance(res, list) else res


def _reject_sys(what, why):
    raise UnsupportedFormError(FVM_ERR_UNSUPPORTED_FORM, f"{what}: {why}; supported system forms are fluxes "
                               "-sum_c D_c(x, y) (alpha[c], beta[c]), sources and Dudt values that are polynomials "
                               "of total degree <= 3 in the components with (x, y) coefficients, Neumann values "
                               "affine in the components, Dirichlet values of (x, y); none may depend on t except for a "
                               "constant term A(x, y) + tau(t) B(x, y), tau(t) = exp(a (t - t0)) or "
                               "1 + a (t - t0) + b (t - t0)^2")


def monomials(N, degree=_SYS_DEGREE):
    """Exponent tuples of the monomials in N variables of total degree <= degree, by degree,
    then lexicographically from the first variable (int8 array (M, N))."""
    out = [()]
    for _ in range(N):
        out = [e + (k,) for e in out for k in range(degree + 1)]
    out = [e for e in out if sum(e) <= degree]
    out.sort(key=lambda e: (sum(e), tuple(-k for k in e)))
    return np.array(out, dtype=np.int8).reshape(-1, N)


def _vandermonde(U, exps):
    return np.prod(U[:, None, :] ** exps[None, :, :].astype(np.float64), axis=2)


def classify_system_flux(q, x, y, t0, N, what="flux_function"):
    """D (N, npoints) of a component flux q(x, y, t, alpha, beta, gamma) = -sum_c D_c(x, y)
    (alpha[c], beta[c]), or reject.  Probes alpha, beta, gamma = unit tuples and zero, then
    verifies one seeded combination at a second time."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    zero = (0.0,) * N

    def unit(c, v=1.0):
        return tuple(v if k == c else 0.0 for k in range(N))

    def ev(a, b, g, t=t0):
        try:
            out = evaluate_tuples(q, x, y, t, a, b, g)
        except Exception as e:  # noqa: BLE001
            _reject_sys(what, f"evaluation failed ({e!r})")
        if not (isinstance(out, tuple) and len(out) == 2):
            _reject_sys(what, "a flux must return (qx, qy)")
        return out

    zx, zy = ev(zero, zero, zero)
    D = np.empty((N, n))
    ok = True
    for c in range(N):
        ax, ay = ev(unit(c), zero, zero)
        bx, by = ev(zero, unit(c), zero)
        gx, gy = ev(zero, zero, unit(c))
        D[c] = -ax
        # every probe output that must vanish, and by + D, against the one tolerance
        worst = np.abs(by + D[c])
        for v in (ay, bx, gx, gy, zx, zy):
            np.maximum(worst, np.abs(v), out=worst)
        ok = ok and bool(np.all(worst <= _RTOL * np.maximum(np.abs(D[c]), 1e-300)))
    if ok and np.all(np.isfinite(D)):
        rng = np.random.default_rng(7)
        A, B, G = (rng.uniform(-2.0, 2.0, N) for _ in range(3))
        cx, cy = ev(tuple(float(v) for v in A), tuple(float(v) for v in B), tuple(float(v) for v in G), t0 + 1.37)
        sc = np.maximum(np.abs(D).sum(axis=0), 1e-300) * 2.0
        ok = (np.all(np.abs(cx + (A[:, None] * D).sum(axis=0)) <= _RTOL * sc)
              and np.all(np.abs(cy + (B[:, None] * D).sum(axis=0)) <= _RTOL * sc))
    else:
        ok = False
    if not ok:
        _reject_sys(what, "not of the form -sum_c D_c(x, y) (alpha[c], beta[c])")
    return D


def classify_system_poly(f, x, y, t0, N, what, max_degree=_SYS_DEGREE, tf=None, time=False):
    """(exps (m, N), coefficients (npoints, m)) of f(x, y, t, u) = sum_m c_m(x, y) prod_c
    u[c]^exps[m][c], a polynomial of total degree <= max_degree in the N-tuple u, or reject.
    time=True allows the constant term to depend on t through one factor (`fit_time_factor`
    over [t0, tf]): then the constant coefficient is the static part A and the result has a
    third item, (TimeFactor, B) or None.

    The closure is evaluated at seeded sample tuples u (the same at every point), the
    coefficients fitted by least squares on the full monomial basis (the constant term exactly,
    from u = 0), the monomials whose coefficients vanish dropped and the rest refitted; the fit
    is then verified at fresh tuples and at a second time to a tolerance of 1e-10 relative to
    sum_m |c_m| |u^e_m| at each point (plus 1e-13 of the largest coefficient per monomial, the
    fit's rounding): a t-dependence or non-polynomial part larger than that is rejected."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    exps = monomials(N, max_degree)
    M = exps.shape[0]
    rng = np.random.default_rng(11)
    U = np.vstack([np.zeros((1, N)), rng.uniform(-1.5, 1.5, size=(M + 5, N))])
    Uc = rng.uniform(-2.0, 2.0, size=(4, N))

    def ev(u, t=t0):
        try:
            v = evaluate_tuples(f, x, y, t, tuple(float(c) for c in u))
        except Exception as e:  # noqa: BLE001
            _reject_sys(what, f"evaluation failed ({e!r})")
        if isinstance(v, tuple) or not np.all(np.isfinite(v)):
            _reject_sys(what, "non-finite or non-scalar values")
        return v

    tfit = fit_time_factor(lambda t: ev(np.zeros(N), t), t0, tf, what) if time else None
    Fv = np.stack([ev(u) for u in U])  # (K, n); U[0] is the zero tuple
    # a closure that does not depend on (x, y) gives identical samples at every point: one fit
    same = n > 0 and bool(np.all(Fv == Fv[:, :1]))
    Fu = Fv[:, :1] if same else Fv
    c0 = Fu[0]  # the constant term is the value at u = 0, exactly (Dirichlet values, constant sources)
    G = Fu[1:] - c0
    rest = exps[1:]  # exps[0] is the constant monomial
    # least squares through the pseudo-inverse of the small sample matrix: one product for all points
    coef = np.linalg.pinv(_vandermonde(U[1:], rest)) @ G if rest.shape[0] else np.zeros((0, Fu.shape[1]))
    cmax = np.max(np.abs(coef), axis=1) if rest.shape[0] else np.zeros(0)
    keep = cmax > 1e-12 * max(np.max(cmax, initial=0.0), np.max(np.abs(c0), initial=0.0), 1e-300)
    rest = rest[keep]
    if rest.shape[0]:
        coef = np.linalg.pinv(_vandermonde(U[1:], rest)) @ G
    else:
        coef = np.zeros((0, Fu.shape[1]))
    # a fitted coefficient that is one value up to rounding at every point (it does not depend
    # on (x, y) while another coefficient does) is set to that one value, so the library can
    # keep it as a scalar.  The test is against the coefficient's own size (a spread within
    # 1e-13 of its largest magnitude): a coefficient that really varies is never flattened,
    # however small it is next to the others.
    for k in range(coef.shape[0]):
        row = coef[k]
        lo, hi = row.min(initial=np.inf), row.max(initial=-np.inf)
        if row.size and hi - lo <= 1e-13 * max(abs(lo), abs(hi)):
            row[:] = np.median(row)
    if np.any(c0 != 0):
        exps = np.vstack([exps[:1], rest])
        coef = np.vstack([c0[None, :], coef])
    else:
        exps = rest
    if same:
        coef = np.repeat(coef, n, axis=1)
    tB = np.zeros(n)
    tau = None
    if tfit is not None:  # constant term A + tau(t) B: the constant coefficient becomes A
        A, tau, tB = tfit
        A = np.where(np.abs(A) <= 1e-13 * np.max(np.abs(tB)), 0.0, A)
        if exps.shape[0] and not np.any(exps[0]):
            coef[0] = A
        else:
            exps = np.vstack([np.zeros((1, N), dtype=exps.dtype), exps])
            coef = np.vstack([A[None, :], coef])
        if not np.any(coef[0]):
            exps, coef = exps[1:], coef[1:]
    scale = np.max(np.abs(coef), axis=0) if exps.shape[0] else np.zeros(n)
    scale = np.maximum(scale, np.max(scale, initial=0.0) * 1e-300 + 1e-300)
    checks = [(u, t0) for u in Uc] + [(U[1], t0 + 1.37), (Uc[0], t0 + 1.37)]
    if tau is not None:
        scale = np.maximum(scale, np.abs(tB))
    for u, t in checks:
        pred = (_vandermonde(u[None, :], exps) @ coef)[0] if exps.shape[0] else np.zeros(n)
        # relative to the size of what is summed: sum_m |c_m| |u^e_m| at each point, plus a
        # floor at the fit's rounding (a few ulps of the largest coefficient per monomial)
        terms = (_vandermonde(np.abs(u)[None, :], exps) @ np.abs(coef))[0] if exps.shape[0] else np.zeros(n)
        if tau is not None:
            pred = pred + tau(t) * tB
            terms = terms + np.abs(tau(t) * tB)
        bound = _RTOL * terms + 1e-13 * scale * (exps.shape[0] + (tau is not None)) * (1.0 + np.max(np.abs(u))) ** max_degree
        if not np.all(np.abs(ev(u, t) - pred) <= bound):
            _reject_sys(what, "depends on t" if t != t0 else
                        f"not a polynomial of total degree <= {max_degree} in the components")
    if time:
        return exps, np.ascontiguousarray(coef.T), (None if tau is None else (tau, tB))
    return exps, np.ascontiguousarray(coef.T)
