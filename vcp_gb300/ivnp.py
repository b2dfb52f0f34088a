"""Interval arithmetic on numpy arrays of doubles (host side of the Emden
verification).

An interval is a pair (lo, hi) of float64 arrays.  Every operation computes
its endpoints in round-to-nearest and then moves each endpoint one ulp
outward (``numpy.nextafter``): a correctly rounded result is within half an
ulp of the exact one, so the widened pair always contains the exact result
of the operation on any points of the operand intervals.  This is looser
than directed rounding by at most one ulp per operation and needs no
rounding-mode switch.
"""
from __future__ import annotations

import numpy as np

_NEG = -np.inf
_POS = np.inf


def down(x):
    return np.nextafter(x, _NEG)


def up(x):
    return np.nextafter(x, _POS)


def point(x):
    x = np.asarray(x, dtype=np.float64)
    return x.copy(), x.copy()


def add(a, b):
    return down(a[0] + b[0]), up(a[1] + b[1])


def sub(a, b):
    return down(a[0] - b[1]), up(a[1] - b[0])


def neg(a):
    return -a[1], -a[0]


def mul(a, b):
    p = (a[0] * b[0], a[0] * b[1], a[1] * b[0], a[1] * b[1])
    lo = np.minimum(np.minimum(p[0], p[1]), np.minimum(p[2], p[3]))
    hi = np.maximum(np.maximum(p[0], p[1]), np.maximum(p[2], p[3]))
    return down(lo), up(hi)


def scale(a, c):
    """a times the exact scalar (or array) c."""
    c = np.asarray(c, dtype=np.float64)
    lo, hi = a[0] * c, a[1] * c
    return down(np.minimum(lo, hi)), up(np.maximum(lo, hi))


def div_exact(a, c):
    """a divided by the exact positive scalar (or array) c."""
    c = np.asarray(c, dtype=np.float64)
    return down(a[0] / c), up(a[1] / c)


def sqr(a):
    lo2, hi2 = a[0] * a[0], a[1] * a[1]
    pos = a[0] >= 0
    negv = a[1] <= 0
    lo = np.where(pos, lo2, np.where(negv, hi2, 0.0))
    hi = np.maximum(lo2, hi2)
    return np.where(lo > 0, down(lo), 0.0), up(hi)


def to_kv(a) -> np.ndarray:
    """Interleave (lo, hi) into the kv layout (flat, same element order)."""
    lo = np.asarray(a[0], dtype=np.float64).ravel(order="K")
    hi = np.asarray(a[1], dtype=np.float64).ravel(order="K")
    out = np.empty(2 * lo.size, dtype=np.float64)
    out[0::2] = lo
    out[1::2] = hi
    return out


def from_kv(buf):
    buf = np.asarray(buf, dtype=np.float64)
    return buf[0::2].copy(), buf[1::2].copy()


def sum_upper(x) -> float:
    """An upper bound of the exact sum of the float64 array x (math.fsum is
    the correctly rounded exact sum)."""
    import math
    return float(up(math.fsum(np.asarray(x, dtype=np.float64).ravel().tolist())))


def sum_lower(x) -> float:
    import math
    return float(down(math.fsum(np.asarray(x, dtype=np.float64).ravel().tolist())))
