"""Krivanek wave aberrations (drop-in for temgym_core.aberrations,
aberrations.py:5-108).

``W_krivanek``, ``grad_W_krivanek`` and ``krivanek_coeff_brackets`` evaluate
the series on NumPy arrays or torch tensors (host / torch-device helpers for
plotting and set-up) from its expansion into monomials of the slopes
(``aberration_monomials``), the same coefficients the fused GPU kernels use
for ``AberratedLensKrivanek``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import astuple, dataclass, fields
from functools import lru_cache

import numpy as np
import torch


@dataclass
class KrivanekCoeffs:
    """aberrations.py:5-31 (same fields, order and defaults)."""
    C10: float = 0.0
    C12: float = 0.0
    phi12: float = 0.0
    C21: float = 0.0
    phi21: float = 0.0
    C23: float = 0.0
    phi23: float = 0.0
    C30: float = 0.0
    C32: float = 0.0
    phi32: float = 0.0
    C34: float = 0.0
    phi34: float = 0.0
    C41: float = 0.0
    phi41: float = 0.0
    C43: float = 0.0
    phi43: float = 0.0
    C45: float = 0.0
    phi45: float = 0.0
    C50: float = 0.0
    C52: float = 0.0
    phi52: float = 0.0
    C54: float = 0.0
    phi54: float = 0.0
    C56: float = 0.0
    phi56: float = 0.0

    def as_list(self) -> list:
        """The 25 values in field order (the C ABI's p[1..25])."""
        return [float(v) for v in astuple(self)]


FIELD_NAMES = tuple(f.name for f in fields(KrivanekCoeffs))


def as_coeffs(c) -> KrivanekCoeffs:
    if isinstance(c, KrivanekCoeffs):
        return c
    if isinstance(c, dict):
        return KrivanekCoeffs(**c)
    raise TypeError("coeffs must be a KrivanekCoeffs or a dict of its fields")


def _lib(v):
    return torch if isinstance(v, torch.Tensor) else np


def _off(D: int, p: int) -> int:
    """Index of the coefficient of x^p y^0 in a degree-D triangle."""
    return p * (D + 1) - p * (p - 1) // 2


@lru_cache(maxsize=64)
def _monomials_cached(kc: tuple):
    from . import _native as N
    a = (C.c_double * 25)(*kc)
    w, gx, gy = (C.c_double * 28)(), (C.c_double * 21)(), (C.c_double * 21)()
    N.check(N.lib().tg_aber_monomials(a, w, gx, gy), "tg_aber_monomials")
    return tuple(w), tuple(gx), tuple(gy)


def aberration_monomials(p):
    """W as a polynomial in the slopes: coefficients of ax^p ay^q of W
    (degree <= 6, triangle order p * 7 - p (p - 1) / 2 + q) and of dW/dax,
    dW/day (degree <= 5).  Every Krivanek term alpha^n cos(m (phi - phi0))
    is |u|^(n-m) Re(u^m e^(-i m phi0)) with u = ax + i ay and n - m even, a
    polynomial; the library expands the series once (tg_aber_monomials), and
    the GPU kernels evaluate the aberrated lens from the same coefficients."""
    w, gx, gy = _monomials_cached(tuple(as_coeffs(p).as_list()))
    return np.array(w), np.array(gx), np.array(gy)


def _tri_eval(c, D: int, x, y):
    """Horner evaluation of a degree-D triangle polynomial (NumPy or torch)."""
    acc = None
    for pp in range(D, -1, -1):
        inner = 0.0 * y
        o = _off(D, pp)
        for qq in range(D - pp, -1, -1):
            inner = inner * y + float(c[o + qq])
        acc = inner if acc is None else acc * x + inner
    return acc


def krivanek_coeff_brackets(phi, p: KrivanekCoeffs):
    """aberrations.py:42-48: the angular brackets B2..B6.  W's degree-n
    homogeneous part is alpha^n B_n / n, so B_n(phi) is n times that part
    evaluated on the unit circle (cos phi, sin phi)."""
    w, _, _ = aberration_monomials(p)
    L = _lib(phi)
    c, s = L.cos(phi), L.sin(phi)
    out = []
    for n in range(2, 7):
        b = 0.0 * c
        for pp in range(n + 1):
            coef = float(w[_off(6, pp) + n - pp])
            if coef != 0.0:
                b = b + coef * c ** pp * s ** (n - pp)
        out.append(n * b)
    return tuple(out)


def W_krivanek(alpha, phi, p):
    """aberrations.py:51-61: W(alpha, phi), as the monomial polynomial at the
    slopes (alpha cos phi, alpha sin phi)."""
    w, _, _ = aberration_monomials(p)
    L = _lib(alpha)
    return _tri_eval(w, 6, alpha * L.cos(phi), alpha * L.sin(phi))


def grad_W_krivanek(alpha_x, alpha_y, p):
    """aberrations.py:64-108: (dW/d alpha_x, dW/d alpha_y), the derivative
    polynomials at the slopes (no polar chain rule, so alpha = 0 needs no
    guard: the gradient there is the polynomials' constant terms, 0)."""
    _, gx, gy = aberration_monomials(p)
    return _tri_eval(gx, 5, alpha_x, alpha_y), _tri_eval(gy, 5, alpha_x, alpha_y)
