"""Host model of the dd GEMM (vcpcu_ddgemm): Python exact integers, used only
by the tests (small sizes).  It restates the same steps as the GPU form --
per-row / per-column exponents one bit above max |a1|, each dd word scaled to
the w-bit grid and rounded to nearest-even separately, the exact integer
product, rounding to dd (hi to nearest, then the exact remainder to nearest)
and the upward-rounded error bound -- so the GPU result must agree bit for
bit.  The reference's pddblas::mulmm (vcp/pddblas.hpp:318-376) computes the
same product approximately (double slices, dd accumulation)."""
from __future__ import annotations

import math
import struct
from fractions import Fraction

MODULI = [256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199, 197, 193,
          191, 181, 179, 173, 167, 163, 157, 151, 149, 139, 137, 131, 127, 113, 109, 107]
ZERO = -30000


def bits_of(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def exponent(amax: float) -> int:
    """E with amax <= 2^(E-1) (E = frexp exponent + 1), ZERO for 0."""
    if amax == 0.0:
        return ZERO
    return math.frexp(amax)[1] + 1


def plan_bits(k: int, slices: int) -> tuple[int, int]:
    w = 8 * slices
    keff = max(k, 1)
    while True:
        need = (2.0 * w - 1.0) + math.log2(keff) + 0.01
        bits, L = 0.0, 0
        while L < len(MODULI) and bits <= need:
            bits += math.log2(MODULI[L])
            L += 1
        if bits > need:
            return w, L
        w -= 1


def scaled_int(x: float, E: int, w: int) -> int:
    """round-half-even(x * 2^(w - E)) exactly."""
    if x == 0.0:
        return 0
    f = Fraction(x) * Fraction(2) ** (w - E)
    q, r = divmod(f.numerator, f.denominator)
    twice = 2 * r
    if twice > f.denominator or (twice == f.denominator and q % 2 == 1):
        q += 1
    return q


def ru(v: Fraction) -> float:
    """Smallest double >= v (v finite, positive range)."""
    d = float(v)
    if Fraction(d) < v:
        d = math.nextafter(d, math.inf)
    return d


def ddgemm(m, n, k, A, B, slices=14):
    """A, B: flat kv dd buffers (column-major).  Returns (C list, err list)."""
    w, _ = plan_bits(k, slices)
    E = []
    for i in range(m):
        am = max([abs(A[2 * (i + p * m)]) for p in range(k)] or [0.0])
        e = exponent(am)
        E.append(e + 1 if e != ZERO else e)
    F = []
    for j in range(n):
        am = max([abs(B[2 * (p + j * k)]) for p in range(k)] or [0.0])
        e = exponent(am)
        F.append(e + 1 if e != ZERO else e)
    Ai = [[(scaled_int(A[2 * (i + p * m)], E[i], w) + scaled_int(A[2 * (i + p * m) + 1], E[i], w))
           if E[i] != ZERO else 0 for p in range(k)] for i in range(m)]
    Bi = [[(scaled_int(B[2 * (p + j * k)], F[j], w) + scaled_int(B[2 * (p + j * k) + 1], F[j], w))
           if F[j] != ZERO else 0 for p in range(k)] for j in range(n)]
    C = [0.0] * (2 * m * n)
    err = [0.0] * (m * n)
    kf = ru(Fraction(max(k, 0)) * (1 + Fraction(1, 2 ** 40)))
    for j in range(n):
        for i in range(m):
            t = i + j * m
            if E[i] == ZERO or F[j] == ZERO:
                continue
            X = sum(a * b for a, b in zip(Ai[i], Bi[j]))
            ex = E[i] + F[j] - 2 * w
            hi = lo = 0.0
            e1 = Fraction(0)
            if X != 0:
                hm = float(X)  # round to nearest
                Y = X - int(Fraction(hm))
                hi = math.ldexp(hm, ex)
                lo = math.ldexp(float(Y), ex) if Y != 0 else 0.0
                e1 = Fraction(ru(Fraction(abs(lo)) * Fraction(1, 2 ** 52) + Fraction(2) ** -1074))
            tr = Fraction(ru(Fraction(kf) * Fraction(2) ** (E[i] + F[j] - w)))
            C[2 * t], C[2 * t + 1] = hi, lo
            err[t] = ru(e1 + tr)
    return C, err
