"""Krivanek wave aberrations (drop-in for temgym_core.aberrations,
aberrations.py:5-108).

``W_krivanek`` and ``grad_W_krivanek`` evaluate the series on NumPy arrays or
torch tensors (host / torch-device helpers for plotting and set-up).  The GPU
ray chain evaluates the same series inside the fused kernels from monomial
coefficients compiled once per component (``AberratedLensKrivanek``).
"""
from __future__ import annotations

from dataclasses import astuple, dataclass, fields

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


def _cos(m, ph, ph0):
    return _lib(ph).cos(m * (ph - ph0))


def _sin(m, ph, ph0):
    return _lib(ph).sin(m * (ph - ph0))


def krivanek_coeff_brackets(phi, p: KrivanekCoeffs):
    """aberrations.py:42-48: the angular brackets B2..B6."""
    B2 = p.C10 + p.C12 * _cos(2, phi, p.phi12)
    B3 = p.C21 * _cos(1, phi, p.phi21) + p.C23 * _cos(3, phi, p.phi23)
    B4 = p.C30 + p.C32 * _cos(2, phi, p.phi32) + p.C34 * _cos(4, phi, p.phi34)
    B5 = p.C41 * _cos(1, phi, p.phi41) + p.C43 * _cos(3, phi, p.phi43) + p.C45 * _cos(5, phi, p.phi45)
    B6 = (p.C50 + p.C52 * _cos(2, phi, p.phi52) + p.C54 * _cos(4, phi, p.phi54)
          + p.C56 * _cos(6, phi, p.phi56))
    return B2, B3, B4, B5, B6


def W_krivanek(alpha, phi, p):
    """aberrations.py:51-61: W(alpha, phi)."""
    p = as_coeffs(p)
    B2, B3, B4, B5, B6 = krivanek_coeff_brackets(phi, p)
    a2 = alpha * alpha
    a3 = a2 * alpha
    a4 = a2 * a2
    a6 = a3 * a3
    return 0.5 * a2 * B2 + (a3 / 3.0) * B3 + 0.25 * a4 * B4 + 0.2 * a4 * alpha * B5 + (a6 / 6.0) * B6


def grad_W_krivanek(alpha_x, alpha_y, p):
    """aberrations.py:64-108: (dW/d alpha_x, dW/d alpha_y) through the polar
    chain rule, with alpha = 0 guarded as in the reference."""
    p = as_coeffs(p)
    L = _lib(alpha_x)
    a = L.hypot(alpha_x, alpha_y) if L is np else torch.hypot(alpha_x, alpha_y)
    phi = L.arctan2(alpha_y, alpha_x)
    B2, B3, B4, B5, B6 = krivanek_coeff_brackets(phi, p)
    a2 = a * a
    a3 = a2 * a
    a4 = a2 * a2
    a5 = a4 * a
    a6 = a3 * a3
    dW_da = a * B2 + a2 * B3 + a3 * B4 + a4 * B5 + a5 * B6
    dW_dphi = (0.5 * a2) * (-2.0 * p.C12 * _sin(2, phi, p.phi12))
    dW_dphi = dW_dphi + (a3 / 3.0) * (-1.0 * p.C21 * _sin(1, phi, p.phi21) - 3.0 * p.C23 * _sin(3, phi, p.phi23))
    dW_dphi = dW_dphi + (0.25 * a4) * (-2.0 * p.C32 * _sin(2, phi, p.phi32) - 4.0 * p.C34 * _sin(4, phi, p.phi34))
    dW_dphi = dW_dphi + (0.2 * a5) * (-1.0 * p.C41 * _sin(1, phi, p.phi41) - 3.0 * p.C43 * _sin(3, phi, p.phi43)
                                      - 5.0 * p.C45 * _sin(5, phi, p.phi45))
    dW_dphi = dW_dphi + (a6 / 6.0) * (-2.0 * p.C52 * _sin(2, phi, p.phi52) - 4.0 * p.C54 * _sin(4, phi, p.phi54)
                                      - 6.0 * p.C56 * _sin(6, phi, p.phi56))
    a_safe = L.where(a == 0, 1e-30, a) if L is np else torch.where(a == 0, torch.full_like(a, 1e-30), a)
    inv_a = 1.0 / a_safe
    inv_a2 = inv_a * inv_a
    dWx = dW_da * (alpha_x * inv_a) + dW_dphi * (-alpha_y * inv_a2)
    dWy = dW_da * (alpha_y * inv_a) + dW_dphi * (alpha_x * inv_a2)
    return dWx, dWy
