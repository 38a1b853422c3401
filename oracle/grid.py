"""FP64 restatement of detector pixel geometry and binning (oracle; tests only).

Follows:
  - ``pixels_to_metres_transform``  coordinate_transforms.py:50-101
    (flip @ flipY @ rotate(deg) @ shift(centre) @ scale @ shift(-(shape-1)/2);
    ``centre`` is passed in (x, y) order to the (y, x) shift, as the
    reference does)
  - ``_rotate``                     coordinate_transforms.py:7-30
  - ``apply_transformation``        coordinate_transforms.py:104-140
  - ``Grid.metres_to_pixels``       grid.py:120-153 (round half-to-even, int32)
  - ``Grid.pixels_to_metres``       grid.py:155-182
  - ``Grid.coords``                 grid.py:83-100 (row-major (x, y) pairs)
  - ``Grid.into_image`` + numba ``inplace_sum``  grid.py:231-280, utils.py:83-114

The 3x3 product ``M @ [y, x, 1]`` is evaluated with the fixed operation order
``(M[i,0]*y + M[i,1]*x) + M[i,2]`` and no fused multiply-add; XLA's dot does
not specify an order, so this is the order the project pins (bit-exactness
is defined against it).  Float->int32 conversion saturates and maps NaN to 0
(XLA's convert semantics).
"""
from __future__ import annotations

import numpy as np


def _rotate(radians):
    c, s = np.cos(radians), np.sin(radians)
    return np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]])


def _scale(p):
    return np.array([[p[0], 0.0, 0.0], [0.0, p[1], 0.0], [0.0, 0.0, 1.0]])


def _shift(c):
    return np.array([[1.0, 0.0, c[0]], [0.0, 1.0, c[1]], [0.0, 0.0, 1.0]])


def _flip_y():
    return np.array([[-1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def pixels_to_metres_transform(centre, pixel_size, shape, flip_y=False, rotation=0.0):
    """coordinate_transforms.py:50-101."""
    flip = _flip_y() if flip_y else np.eye(3)
    shape = np.asarray(shape, dtype=np.float64)
    pixel_shift = _shift(-(shape - 1) / 2.0)
    scale = _scale(pixel_size)
    centre_shift = _shift(centre)
    rot = _rotate(np.pi / 180 * rotation)
    return flip @ _flip_y() @ rot @ centre_shift @ scale @ pixel_shift


def metres_to_pixels_mat(centre, pixel_size, shape, flip_y=False, rotation=0.0):
    """grid.py:51-63 (inverse of the pixels->metres transform)."""
    return np.linalg.inv(pixels_to_metres_transform(centre, pixel_size, shape, flip_y, rotation))


def _apply(m, a, b):
    """coordinate_transforms.py:137-140 with the pinned operation order."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    o0 = (m[0, 0] * a + m[0, 1] * b) + m[0, 2]
    o1 = (m[1, 0] * a + m[1, 1] * b) + m[1, 2]
    return o0, o1


def round_to_int32(v):
    """jnp.round (half-to-even) then astype(int32), saturating, NaN -> 0."""
    v = np.rint(np.asarray(v, dtype=np.float64))
    out = np.where(np.isnan(v), 0.0, v)
    out = np.clip(out, -2147483648.0, 2147483647.0)
    return out.astype(np.int32)


def metres_to_pixels(grid: dict, x, y, cast=True):
    """grid.py:120-153.  Returns (py, px)."""
    m = metres_to_pixels_mat(grid.get("centre", (0.0, 0.0)), grid["pixel_size"], grid["shape"],
                             grid.get("flip_y", False), grid.get("rotation", 0.0))
    py, px = _apply(m, y, x)
    if cast:
        return round_to_int32(py), round_to_int32(px)
    return py, px


def pixels_to_metres(grid: dict, py, px):
    """grid.py:155-182.  Returns (x, y) in metres."""
    t = pixels_to_metres_transform(grid.get("centre", (0.0, 0.0)), grid["pixel_size"],
                                   grid["shape"], grid.get("flip_y", False),
                                   grid.get("rotation", 0.0))
    my, mx = _apply(t, py, px)
    return mx, my


def grid_coords(grid: dict):
    """grid.py:83-100: (H*W, 2) pixel-centre (x, y) pairs, row-major."""
    h, w = grid["shape"]
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    x, y = pixels_to_metres(grid, yy.ravel(), xx.ravel())
    return np.stack((x, y), axis=-1)


def into_image(grid: dict, py, px, acc=None, mask=None):
    """grid.py:231-280 + utils.py:83-114: acc[py, px] += 1 for in-bounds hits."""
    h, w = grid["shape"]
    if acc is None:
        acc = np.zeros((h, w), dtype=np.int64)
    py = np.asarray(py).ravel()
    px = np.asarray(px).ravel()
    ok = (py >= 0) & (py < h) & (px >= 0) & (px < w)
    if mask is not None:
        ok &= np.asarray(mask, dtype=bool).ravel()
    np.add.at(acc, (py[ok], px[ok]), 1)
    return acc
