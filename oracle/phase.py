"""Exact reduction of k*pathlength modulo 2*pi (oracle; tests only).

The reference forms ``phase_offset = k * pathlength`` in float64
(gaussian.py:253-255) and adds it to the per-pixel phase (gaussian.py:316).
At k = 2*pi/1.97e-12 m and pathlength ~ 1 m that product is ~3.2e12 rad,
whose float64 spacing is ~4.9e-4 rad, so the reference-literal value carries
rounding of that size.  The oracle instead reduces the EXACT product of the
two given float64 numbers:

  * TwoProduct without FMA, by Dekker's splitting (T. J. Dekker, "A
    floating-point technique for extending the available precision",
    Numer. Math. 18, 1971): k*pl = p + e exactly.
  * Cody-Waite style reduction by a double-double 2*pi = C1 + C2, with
    n*C1 formed exactly by TwoProduct again.

Result: the reduced phase in [-pi, pi] with error ~1e-15 rad.
"""
from __future__ import annotations

import numpy as np

_SPLIT = 134217729.0  # 2**27 + 1
TWO_PI_HI = 6.283185307179586  # fl(2*pi)
TWO_PI_LO = 2.4492935982947064e-16  # 2*pi - fl(2*pi)


def _split(a):
    c = _SPLIT * a
    hi = c - (c - a)
    return hi, a - hi


def two_prod(a, b):
    """Exact a*b = p + e (Dekker), elementwise float64."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def reduce_2pi_dd(p, e=0.0):
    """(p + e) mod 2*pi into [-pi, pi], for a double-double input."""
    p = np.asarray(p, dtype=np.float64)
    n = np.rint(p / TWO_PI_HI)
    q, qe = two_prod(n, TWO_PI_HI)
    r = (p - q)  # exact: q is within a factor 2 of p (Sterbenz)
    r = r + ((e - qe) - n * TWO_PI_LO)
    # one more wrap in case rounding pushed r just outside [-pi, pi]
    r = np.where(r > np.pi, r - 2 * np.pi, np.where(r < -np.pi, r + 2 * np.pi, r))
    return r


def phase_offset_exact(k, pathlength):
    """k * pathlength mod 2*pi, from the exact product of the float64 inputs."""
    p, e = two_prod(k, pathlength)
    return reduce_2pi_dd(p, e)


def wrap(phi):
    """Wrap angles to (-pi, pi]."""
    return np.angle(np.exp(1j * np.asarray(phi)))
