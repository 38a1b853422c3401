"""Pixel <-> metre homogeneous transforms (coordinate_transforms.py:7-140).

Host float64 set-up math (3x3 matrices); the per-ray application runs on the
GPU (tg_bin / tg_trace_fwd).
"""
from __future__ import annotations

import numpy as np


def _rotate(radians: float) -> np.ndarray:
    """coordinate_transforms.py:17-30 (y-axis flipped convention)."""
    c, s = np.cos(radians), np.sin(radians)
    return np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]], dtype=np.float64)


def _scale(pixel_size_yx) -> np.ndarray:
    return np.array([[pixel_size_yx[0], 0.0, 0.0], [0.0, pixel_size_yx[1], 0.0],
                     [0.0, 0.0, 1.0]], dtype=np.float64)


def _shift(c) -> np.ndarray:
    return np.array([[1.0, 0.0, c[0]], [0.0, 1.0, c[1]], [0.0, 0.0, 1.0]], dtype=np.float64)


def _flip_y() -> np.ndarray:
    return np.array([[-1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]], dtype=np.float64)


def pixels_to_metres_transform(centre, pixel_size, shape, flip_y=False, rotation=0.0):
    """coordinate_transforms.py:50-101:
    flip @ flipY @ rotate(deg) @ shift(centre) @ scale(pixel_size) @ shift(-(shape-1)/2).
    ``centre`` is given as (x, y) and enters the (y, x) shift as-is, exactly
    as the reference passes it."""
    flip = _flip_y() if flip_y else np.eye(3)
    shape = np.asarray(shape, dtype=np.float64)
    return (flip @ _flip_y() @ _rotate(np.pi / 180 * float(rotation))
            @ _shift(tuple(float(v) for v in centre))
            @ _scale(tuple(float(v) for v in pixel_size)) @ _shift(-(shape - 1) / 2.0))


def metres_to_pixels_transform(centre, pixel_size, shape, flip_y=False, rotation=0.0):
    """grid.py:51-63: inverse (LU) of the pixels->metres transform."""
    return np.linalg.inv(pixels_to_metres_transform(centre, pixel_size, shape, flip_y, rotation))


def apply_transformation(y, x, transformation):
    """coordinate_transforms.py:104-140: [y', x', 1] = T [y, x, 1] for every
    coordinate pair (any matching shapes).  Torch tensors stay on their
    device; anything else is computed with NumPy in float64.  The per-ray
    binning on the path does not come here: it runs in the GPU binner
    (tg_bin / tg_trace_fwd), bit-exact with this float64 arithmetic."""
    import torch
    if isinstance(y, torch.Tensor) or isinstance(x, torch.Tensor):
        dev = y.device if isinstance(y, torch.Tensor) else x.device
        t = torch.as_tensor(np.asarray(transformation, dtype=np.float64), device=dev)
        yt = torch.as_tensor(y, dtype=torch.float64, device=dev)
        xt = torch.as_tensor(x, dtype=torch.float64, device=dev)
        yt, xt = torch.broadcast_tensors(yt, xt)
        return ((t[0, 0] * yt + t[0, 1] * xt) + t[0, 2], (t[1, 0] * yt + t[1, 1] * xt) + t[1, 2])
    t = np.asarray(transformation, dtype=np.float64)
    yy, xx = np.broadcast_arrays(np.asarray(y, np.float64), np.asarray(x, np.float64))
    return (t[0, 0] * yy + t[0, 1] * xx) + t[0, 2], (t[1, 0] * yy + t[1, 1] * xx) + t[1, 2]
