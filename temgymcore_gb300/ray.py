"""Ray records (drop-in for temgym_core ``Ray`` ray.py:8-166 and
``GaussianRay`` gaussian.py:113-177).

Fields hold Python floats, NumPy arrays or torch tensors.  The device layout
used by the kernels is a structure of arrays: x, y, dx, dy as contiguous
float32 CUDA tensors, pathlength as float64 (per ray or one uniform value),
z as one uniform float64 value or a per-ray float64 tensor.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from .tree_utils import HasParamsMixin


def _size(v) -> int:
    if isinstance(v, torch.Tensor):
        return int(v.numel()) if v.dim() > 0 else 1
    if isinstance(v, np.ndarray):
        return int(v.size) if v.ndim > 0 else 1
    return 1


def _is_vec(v) -> bool:
    return (isinstance(v, (torch.Tensor, np.ndarray)) and v.ndim > 0)


@dataclass(frozen=True)
class Ray(HasParamsMixin):
    """Parametric ray(s): positions x, y (m), slopes dx, dy (rad), axial z (m),
    accumulated pathlength (m) and the homogeneous carrier ``_one``
    (ray.py:8-45).  Vector rays hold 1-D arrays of equal length."""

    x: Any
    y: Any
    dx: Any
    dy: Any
    z: Any
    pathlength: Any
    _one: Any = 1.0

    @classmethod
    def origin(cls):
        """ray.py:48-57."""
        return cls(*((0.0,) * 6))

    @property
    def size(self) -> int:
        """ray.py:59-77 (asserts equal field sizes)."""
        cached = self.__dict__.get("_size_cache")  # fields are frozen: computed once
        if cached is not None:
            return cached
        sizes = {_size(getattr(self, f.name)) for f in dataclasses.fields(self)
                 if _is_vec(getattr(self, f.name))}
        assert len(sizes) <= 1, "ray fields have mismatched sizes"
        n = sizes.pop() if sizes else 1
        object.__setattr__(self, "_size_cache", n)
        return n

    def __getitem__(self, arg):
        """ray.py:79-96."""
        return type(self)(**{f.name: (getattr(self, f.name)[arg] if _is_vec(getattr(self, f.name))
                                      else getattr(self, f.name))
                             for f in dataclasses.fields(self)})

    def to_ray(self):
        return self

    def item(self):
        """ray.py:98-117: single-element ray to Python scalars."""
        out = {}
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            out[f.name] = v.item() if hasattr(v, "item") and _size(v) == 1 else v
        return type(self)(**out)

    def to_vector(self):
        """ray.py:119-125."""
        out = {}
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, torch.Tensor):
                out[f.name] = v.reshape(-1)
            else:
                out[f.name] = np.atleast_1d(np.asarray(v))
        return type(self)(**out)

    def derive(self, x=None, y=None, dx=None, dy=None, z=None, pathlength=None):
        """ray.py:127-166: modified copy (``_one`` preserved)."""
        return dataclasses.replace(
            self,
            x=self.x if x is None else x, y=self.y if y is None else y,
            dx=self.dx if dx is None else dx, dy=self.dy if dy is None else dy,
            z=self.z if z is None else z,
            pathlength=self.pathlength if pathlength is None else pathlength)


@dataclass(frozen=True, kw_only=True)
class GaussianRay(Ray):
    """Gaussian beamlet: a central ray plus complex amplitude, waist (x, y),
    radii of curvature (x, y), wavelength and rotation theta (rad)
    (gaussian.py:113-177)."""

    amplitude: Any
    waist_xy: Any
    radii_of_curv: Any
    wavelength: Any
    theta: Any

    def to_ray(self) -> Ray:
        return Ray(x=self.x, y=self.y, dx=self.dx, dy=self.dy, z=self.z,
                   pathlength=self.pathlength, _one=self._one)

    @property
    def size(self) -> int:
        """Number of beams: per-beam fields have length n; waist_xy and
        radii_of_curv are (n, 2)."""
        sizes = set()
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if not _is_vec(v):
                continue
            if f.name in ("waist_xy", "radii_of_curv"):
                sizes.add(int(np.shape(v)[0]) if np.ndim(v) == 2 else 1)
            else:
                sizes.add(_size(v))
        sizes.discard(1) if len(sizes) > 1 else None
        assert len(sizes) <= 1, "beam fields have mismatched sizes"
        return sizes.pop() if sizes else 1

    def derive(self, **updates):
        return dataclasses.replace(self, **{k: (v(self) if callable(v) else v)
                                            for k, v in updates.items()})

    @property
    def q_inv(self):
        """(1/qx, 1/qy) on the principal axes, complex128 on the device
        (gaussian.py:138-157): i wavelength / (pi w^2), minus 1/R where the
        radius is finite."""
        from .gaussian import beam_q_inv
        return beam_q_inv(self, full=False)

    @property
    def Q_inv(self):
        """(n, 2, 2) complex128 R(theta) diag(1/qx, 1/qy) R(theta)^T on the
        device (gaussian.py:159-177)."""
        from .gaussian import beam_q_inv
        return beam_q_inv(self, full=True)


# ------------------------------------------------------------- device layout

def _dev():
    return torch.device("cuda", torch.cuda.current_device())


def as_f32(v, n: int, device) -> torch.Tensor:
    """Contiguous float32 device vector of length n (broadcasting scalars)."""
    if (isinstance(v, torch.Tensor) and v.dtype == torch.float32 and v.dim() == 1 and v.is_cuda
            and v.numel() == n and v.is_contiguous() and v.device == device):
        return v  # already in the kernel layout (only its address is used)
    if isinstance(v, torch.Tensor):
        t = v.detach().to(device=device, dtype=torch.float32).reshape(-1)
    else:
        t = torch.as_tensor(np.asarray(v, dtype=np.float32).reshape(-1), device=device)
    if t.numel() == 1 and n != 1:
        t = t.expand(n)
    return t.contiguous()


def as_f64_or_scalar(v, n: int, device):
    """(tensor or None, scalar): per-ray float64 vector, or one uniform value."""
    if isinstance(v, torch.Tensor):
        if v.numel() == 1 and v.dim() == 0:
            return None, float(v.detach().item())
        t = v.detach().to(device=device, dtype=torch.float64).reshape(-1)
        if t.numel() == 1 and n != 1:
            return None, float(t.item())
        return t.contiguous(), 0.0
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 0 or (a.size == 1 and n != 1):
        return None, float(a.reshape(-1)[0])
    return torch.as_tensor(a.reshape(-1), device=device).contiguous(), 0.0


def is_uniform(v) -> bool:
    """True when a z / pathlength field holds a single value for all rays."""
    if isinstance(v, torch.Tensor):
        return v.dim() == 0
    return np.asarray(v).ndim == 0
