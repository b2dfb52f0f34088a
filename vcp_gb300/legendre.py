"""Rigorous tables of VCP's Legendre basis at Gauss-Legendre points.

The Legendre_Bases_Generator of the reference (vcp/ldbase.hpp) works with
the one-dimensional basis

    phi_i(t) = t (1 - t) P~'_{i-1}(t) / (i (i - 1)),   i = 2 .. M + 1

on [0, 1] (makeLegendreBase, vcp/ldbase.hpp:155-181; P~_n the Legendre
polynomials shifted to [0, 1], NmalLegendrePol :130-153), and evaluates it at
the Gauss-Legendre points of [0, 1] (setting, :672-831: nodes (x + 1) / 2 and
weights w / 2 of the rule on [-1, 1]) in interval<mpfr<500>> arithmetic
before converting the values to the matrix type.

This module computes the same tables with mpmath's interval arithmetic
(``mpmath.iv``), which rounds every operation outward, and converts them to
double intervals by outward rounding:

* nodes: the roots of P_n on [-1, 1], refined by Newton's method, each
  enclosed in X = [x - d, x + d] with d = 1e-38 and the enclosure proved by
  a strict sign change of P_n at its two ends (evaluated in iv); n sign
  changes in n disjoint intervals account for every root;
* weights: w = 2 / ((1 - X^2) P'_n(X)^2) over the node enclosure X, halved
  for [0, 1];
* basis: with s = 2 t - 1, phi_i(t) = -int_0^t P~_{i-1} =
  (P_{i-2}(s) - P_i(s)) / (2 (2 i - 1)) and phi_i''(t) = -2 P'_{i-1}(s).

The three-term recurrences of P_k and P'_k run in iv at the node midpoint x
with 120 digits (run on an interval, the recurrence would widen it about
threefold per step); the values over X follow from the mean-value bounds
|P'_k| <= k (k + 1) / 2 and |P''_k| <= (k - 1) k (k + 1) (k + 2) / 8 on
[-1, 1].

Row a of each (M x npts) table holds phi_{a+2} -- the reference's basis index
a (Legendre_with_GLpoint, :804-818).  Tables are cached in the directory
named by VCP_TABLE_CACHE (default: ``_tables`` beside this file) as .npz.
"""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np

_CACHE = Path(os.environ.get("VCP_TABLE_CACHE", Path(__file__).resolve().parent / "_tables"))
_VERSION = 1


def _mp():
    try:
        import mpmath
    except ImportError as e:  # pragma: no cover - mpmath ships with torch's sympy
        raise RuntimeError("the Legendre tables need mpmath (interval arithmetic)") from e
    return mpmath


def _to_double_down(mpmath, x) -> float:
    f = float(x)
    if mpmath.mpf(f) > x:
        f = float(np.nextafter(f, -np.inf))
    return f


def _to_double_up(mpmath, x) -> float:
    f = float(x)
    if mpmath.mpf(f) < x:
        f = float(np.nextafter(f, np.inf))
    return f


def _outward(mpmath, v) -> tuple[float, float]:
    """Outward double enclosure of the iv interval v (its endpoints are
    binary floats of iv's precision; mp runs at a higher one, so mpf() holds
    them exactly)."""
    return (_to_double_down(mpmath, mpmath.mpf(v.a._mpi_[0])),
            _to_double_up(mpmath, mpmath.mpf(v.b._mpi_[1])))


def _mpf_mid(mpmath, v):
    return mpmath.mpf(v.mid._mpi_[0])


def _pd_point(x, K: int):
    """P_0..P_K and P'_0..P'_K at the point x (an mpf), in iv arithmetic.
    The three-term recurrence widens intervals by about a factor 3 per
    step when run on intervals, so it runs on the point x at a working
    precision (_IV_DPS digits) that leaves the K-step result far below the
    double resolution; an interval argument is handled by the mean-value
    bounds of _widen."""
    iv = _mp().iv
    X = iv.mpf(x)
    one = iv.mpf(1)
    P = [one, X]
    D = [0 * one, one]
    for k in range(1, K):
        P.append(((2 * k + 1) * X * P[k] - k * P[k - 1]) / (k + 1))
        D.append(D[k - 1] + (2 * k + 1) * P[k])
    return P[:K + 1], D[:K + 1]


def _widen(P, D, delta):
    """Enclosures of P_k and P'_k over [x - delta, x + delta] (inside [-1, 1])
    from their values at x: |P'_k| <= k (k + 1) / 2 and
    |P''_k| <= (k - 1) k (k + 1) (k + 2) / 8 on [-1, 1] (the derivatives of
    Legendre polynomials peak at the end points)."""
    iv = _mp().iv
    dl = iv.mpf([-delta, delta])
    Pw = [p + dl * (k * (k + 1) // 2) for k, p in enumerate(P)]
    Dw = [d + dl * iv.mpf((k - 1) * k * (k + 1) * (k + 2)) / 8 if k >= 1 else d
          for k, d in enumerate(D)]
    return Pw, Dw


_IV_DPS = 120


def _setup_precision():
    mpmath = _mp()
    mpmath.iv.dps = _IV_DPS
    mpmath.mp.prec = mpmath.iv.prec + 32
    return mpmath


def gauss_legendre_iv(npts: int):
    """Interval enclosures (mpmath.iv) of the npts Gauss-Legendre nodes and
    weights on [-1, 1], nodes ascending, with the node midpoints (mpf) and
    the half width delta of every node enclosure."""
    mpmath = _setup_precision()
    iv = mpmath.iv
    x0, _ = np.polynomial.legendre.leggauss(npts)
    nodes, weights, mids = [], [], []
    delta = mpmath.mpf(10) ** -38
    prev_hi = None
    for xd in x0:
        x = mpmath.mpf(xd)
        for _ in range(10):
            P, D = _pd_point(x, npts)
            x = x - _mpf_mid(mpmath, P[npts]) / _mpf_mid(mpmath, D[npts])
        a, b = x - delta, x + delta
        pa = _pd_point(a, npts)[0][npts]
        pb = _pd_point(b, npts)[0][npts]
        sa = 1 if pa.a > 0 else (-1 if pa.b < 0 else 0)
        sb = 1 if pb.a > 0 else (-1 if pb.b < 0 else 0)
        if sa == 0 or sb == 0 or sa == sb:
            raise RuntimeError(f"Gauss-Legendre node {xd} of {npts} points not isolated")
        if prev_hi is not None and not (a > prev_hi):
            raise RuntimeError("Gauss-Legendre node enclosures overlap")
        prev_hi = b
        X = iv.mpf([a, b])
        P, D = _pd_point(x, npts)
        _, Dw = _widen(P, D, delta)
        W = 2 / ((1 - X * X) * Dw[npts] * Dw[npts])
        nodes.append(X)
        weights.append(W)
        mids.append(x)
    return nodes, weights, mids, delta


def basis_tables(M: int, npts: int, use_cache: bool = True) -> dict:
    """Double-interval tables of the M basis functions phi_2..phi_{M+1} and
    their second derivatives at the npts Gauss-Legendre points of [0, 1].

    Keys (float64): x_lo, x_hi, w_lo, w_hi (npts); phi_lo, phi_hi,
    dd_lo, dd_hi (M x npts, row a = phi_{a+2}); x_mid, w_mid, phi_mid,
    dd_mid (nearest doubles of the high-precision values)."""
    path = _CACHE / f"legendre_M{M}_n{npts}_v{_VERSION}.npz"
    if use_cache and path.exists():
        with np.load(path) as z:
            return {k: z[k] for k in z.files}
    nodes, weights, mids, delta = gauss_legendre_iv(npts)
    mpmath = _setup_precision()
    out = {k: np.empty(npts) for k in ("x_lo", "x_hi", "w_lo", "w_hi", "x_mid", "w_mid")}
    for k in ("phi_lo", "phi_hi", "dd_lo", "dd_hi", "phi_mid", "dd_mid"):
        out[k] = np.empty((M, npts))
    for q, (X, W, x) in enumerate(zip(nodes, weights, mids)):
        T = (X + 1) / 2
        Wt = W / 2
        out["x_lo"][q], out["x_hi"][q] = _outward(mpmath, T)
        out["w_lo"][q], out["w_hi"][q] = _outward(mpmath, Wt)
        out["x_mid"][q] = float(_mpf_mid(mpmath, T))
        out["w_mid"][q] = float(_mpf_mid(mpmath, Wt))
        P, D = _widen(*_pd_point(x, M + 1), delta)   # P_0..P_{M+1}, P'_0..P'_{M+1} over X
        for a in range(M):
            i = a + 2
            phi = (P[i - 2] - P[i]) / (2 * (2 * i - 1))
            dd = -2 * D[i - 1]
            out["phi_lo"][a, q], out["phi_hi"][a, q] = _outward(mpmath, phi)
            out["dd_lo"][a, q], out["dd_hi"][a, q] = _outward(mpmath, dd)
            out["phi_mid"][a, q] = float(_mpf_mid(mpmath, phi))
            out["dd_mid"][a, q] = float(_mpf_mid(mpmath, dd))
    if use_cache:
        try:
            _CACHE.mkdir(parents=True, exist_ok=True)
            tmp = path.with_suffix(".tmp.npz")
            np.savez(tmp, **out)
            os.replace(tmp, path)
        except OSError:
            pass
    return out


def basis_at_points(M: int, t: np.ndarray, cache_key: str | None = None):
    """Double-interval enclosures of phi_2..phi_{M+1} at the points t of
    [0, 1] (doubles, taken as exact): s = 2 t - 1 is exact in double, the
    recurrences run in iv at s.  Returns (lo, hi), each (M x len(t)); with
    cache_key, cached like the Gauss tables under that name."""
    t = np.asarray(t, dtype=np.float64)
    path = _CACHE / f"points_{cache_key}_M{M}_n{t.size}_v{_VERSION}.npz" if cache_key else None
    if path is not None and path.exists():
        with np.load(path) as z:
            if np.array_equal(z["t"], t):
                return z["lo"], z["hi"]
    lo, hi = _basis_at_points(M, t)
    if path is not None:
        try:
            _CACHE.mkdir(parents=True, exist_ok=True)
            tmp = path.with_suffix(".tmp.npz")
            np.savez(tmp, t=t, lo=lo, hi=hi)
            os.replace(tmp, path)
        except OSError:
            pass
    return lo, hi


def _basis_at_points(M: int, t: np.ndarray):
    mpmath = _setup_precision()
    lo = np.empty((M, t.size))
    hi = np.empty_like(lo)
    for q, tq in enumerate(t):
        P, _ = _pd_point(mpmath.mpf(2.0 * float(tq) - 1.0), M + 1)
        for a in range(M):
            i = a + 2
            lo[a, q], hi[a, q] = _outward(mpmath, (P[i - 2] - P[i]) / (2 * (2 * i - 1)))
    return lo, hi
