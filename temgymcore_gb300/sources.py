"""Ray sources on the GPU (drop-in for source.py:36-188 and utils.py:117-202).

``PointSource(...).generate_array(num)`` / ``ParallelBeam(...).make_rays(num)``
and ``concentric_rings`` / ``random_coords`` write the reference's ray layout
directly into device memory (``csrc/source.cu``).  Deterministic mode
reproduces the reference's concentric rings ray for ray; random mode draws
from the same distribution (uniform in the disc) with a seeded device hash,
not from NumPy's global generator, and returns exactly ``num`` rays.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _native as N
from .run import _device

N.register("tg_source_count", C.c_int, [C.c_int64, C.c_int32, C.POINTER(C.c_int64)])
N.register("tg_source_generate", C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_uint64, C.c_double,
                                           C.c_double, C.c_double, C.c_void_p, C.c_int64, C.c_void_p])

POINT, PARALLEL = 0, 1


def source_count(num: int, random: bool = False) -> int:
    n = C.c_int64(0)
    N.check(N.lib().tg_source_count(int(num), int(bool(random)), C.byref(n)), "tg_source_count")
    return int(n.value)


def generate(kind: int, num: int, extent: float, offset_xy=(0.0, 0.0), random: bool = False,
             seed: int = 0) -> torch.Tensor:
    """(N, 5) float64 device rays [x, y, dx, dy, 1]."""
    dev = _device()
    n = source_count(num, random)
    out = torch.empty((n, 5), dtype=torch.float64, device=dev)
    ox, oy = (float(v) for v in offset_xy)
    N.check(N.lib().tg_source_generate(kind, int(bool(random)), int(num), int(seed) & (2 ** 64 - 1),
                                       float(extent), ox, oy, out.data_ptr(), n, N.stream_ptr()),
            "tg_source_generate")
    return out


def concentric_rings(num_points_approx: int, radius: float) -> torch.Tensor:
    """utils.py:117-175: (N, 2) float64 (y, x) points on concentric rings."""
    r = generate(PARALLEL, num_points_approx, radius)
    return torch.stack((r[:, 1], r[:, 0]), dim=-1)


def random_coords(num: int, seed: int = 0) -> torch.Tensor:
    """utils.py:178-202: (N, 2) float64 (y, x) points uniform in the unit disc."""
    r = generate(PARALLEL, num, 1.0, random=True, seed=seed)
    return torch.stack((r[:, 1], r[:, 0]), dim=-1)
