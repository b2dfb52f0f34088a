"""Seeded synthetic matrices with the distributions of the benchmark configs.

* ``ephi(rng, size, phi)`` -- entries with mantissa uniform in [1, 2), random
  sign and integer exponent uniform in [-phi, phi] (cancellation-heavy for
  large phi).
* ``interval_ephi(rng, rows, cols, phi, rad_ratio)`` -- kv-layout interval
  matrix with midpoints from ``ephi`` and radius ``rad_ratio * |mid|``
  (the n=512 / n=8192 interval workloads use phi = 4, rad_ratio = 2^-40).
* ``interval_uniform(rng, rows, cols, rad_ratio)`` -- midpoints uniform in
  [-1, 1] (the batched workload: rad_ratio = 1e-12).

All matrices are column-major flat float64 arrays.  The endpoints of each
interval are mid -/+ rad rounded to nearest; only their values matter.
"""
from __future__ import annotations

import numpy as np


def ephi(rng: np.random.Generator, size: int, phi: int) -> np.ndarray:
    mant = rng.uniform(1.0, 2.0, size)
    sign = rng.choice(np.array([-1.0, 1.0]), size)
    ex = rng.integers(-phi, phi + 1, size) if phi > 0 else np.zeros(size, dtype=np.int64)
    return sign * np.ldexp(mant, ex)


def _kv(mid: np.ndarray, rad: np.ndarray) -> np.ndarray:
    out = np.empty(2 * mid.size, dtype=np.float64)
    out[0::2] = mid - rad
    out[1::2] = mid + rad
    return out


def interval_ephi(rng, rows: int, cols: int, phi: int = 4,
                  rad_ratio: float = 2.0 ** -40) -> np.ndarray:
    mid = ephi(rng, rows * cols, phi)
    return _kv(mid, np.abs(mid) * rad_ratio)


def interval_uniform(rng, rows: int, cols: int, rad_ratio: float = 1e-12) -> np.ndarray:
    mid = rng.uniform(-1.0, 1.0, rows * cols)
    return _kv(mid, np.abs(mid) * rad_ratio)
