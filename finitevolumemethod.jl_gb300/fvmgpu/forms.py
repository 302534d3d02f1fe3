"""Closures -> device-coded forms.

Julia (and Python) closures are opaque to the GPU.  The host evaluates each closure at the
points where the reference would evaluate it (vertices, dual-edge midpoints, boundary
quarter points) and classifies it:

* a closure of (x, y) alone is sampled into a per-point array;
* a closure that is a polynomial of degree <= 2 in u with (x, y)-dependent coefficients
  becomes the coefficient arrays c0, c1, c2 (f = c0 + c1 u + c2 u^2);
* anything else (t dependence, non-polynomial u dependence, non-finite values) is rejected
  with `UnsupportedFormError`: never guessed.

Classification probes the closure at u in {0, 1, -1} and t in {t0, t0 + 1.37}, fits the
quadratic, and verifies it at u in {2, -0.5, 3.25} and at the second time, to a relative
tolerance of 1e-10.
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
                               "and polynomials of degree <= 2 in u with (x, y) coefficients, independent of t")


def classify_xytu(f, x, y, t0, what, max_degree=2):
    """Coefficients (c0, c1, c2)[:deg+1] and degree of g(x, y, t, u) = f(x, y, t, u) at points."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    t1 = float(t0)
    t2 = t1 + 1.37
    try:
        g = {u: evaluate(f, x, y, t1, np.full(x.shape, u)) for u in _FIT_U}
    except Exception as e:  # noqa: BLE001
        _reject(what, f"evaluation failed ({e!r})")
    for v in g.values():
        if not np.all(np.isfinite(v)):
            _reject(what, "non-finite values")
    c0 = g[0.0]
    c1 = (g[1.0] - g[-1.0]) / 2
    c2 = (g[1.0] + g[-1.0]) / 2 - c0
    scale = np.maximum(np.maximum(np.abs(c0), np.abs(c1)), np.abs(c2))
    scale = np.maximum(scale, np.max(scale) * 1e-300 + 1e-300)
    for u in _CHECK_U:
        gu = evaluate(f, x, y, t1, np.full(x.shape, u))
        pred = c0 + u * (c1 + u * c2)
        if not np.all(np.abs(gu - pred) <= _RTOL * (scale * (1 + abs(u)) ** 2)):
            _reject(what, "not a polynomial of degree <= 2 in u")
    for u in _FIT_U:
        gt = evaluate(f, x, y, t2, np.full(x.shape, u))
        if not np.all(np.abs(gt - g[u]) <= _RTOL * (scale * (1 + abs(u)) ** 2)):
            _reject(what, "depends on t")
    tiny = 1e-14 * np.max(scale) if scale.size else 0.0
    if np.all(np.abs(c2) <= tiny):
        c2 = np.zeros_like(c2)
        if np.all(np.abs(c1) <= tiny):
            c1 = np.zeros_like(c1)
    deg = 2 if np.any(c2 != 0) else (1 if np.any(c1 != 0) else 0)
    if deg > max_degree:
        _reject(what, f"degree {deg} in u exceeds {max_degree}")
    coeffs = np.stack([c0, c1, c2][: deg + 1], axis=-1)
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


def sample_xy(f, x, y, *extra, what="function"):
    """Values of a closure of (x, y[, extra...]) at points (template closures, ICs)."""
    try:
        v = evaluate(f, x, y, *extra)
    except Exception as e:  # noqa: BLE001
        _reject(what, f"evaluation failed ({e!r})")
    if not np.all(np.isfinite(v)):
        _reject(what, "non-finite values")
    return v
