"""Transfer-matrix helpers (drop-in for temgym_core.transfer, transfer.py:6-183).

``transfer_rays`` (in double-float arithmetic: float32 pairs with exact
product errors, results within 1e-13 of the sum of the term magnitudes;
float64 for values outside [2^-39, 2^62]) and ``transfer_rays_pt_src``
(float64) run on the GPU (``csrc/transfer.cu``); ``accumulate_matrices`` and
``accumulate_matrices_cumulative`` are host float64 products of a few 5x5
matrices (the latter through the C ABI, in the reference's order).
Outputs are float64 CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .run import _device

N.register("tg_transfer_cumulative", C.c_int, [C.c_int32, C.c_void_p, C.c_void_p])
N.register("tg_transfer_rays", C.c_int, [C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                         C.c_void_p])
N.register("tg_transfer_rays_pt_src", C.c_int, [C.c_double, C.c_double, C.c_int64, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p])


def _host_mats(m) -> np.ndarray:
    if isinstance(m, torch.Tensor):
        m = m.detach().cpu().numpy()
    a = np.ascontiguousarray(np.asarray(m, dtype=np.float64))
    if a.ndim != 3 or a.shape[1:] != (5, 5):
        raise ValueError("transfer matrices must have shape (M, 5, 5)")
    return a


def _dev64(v, dev) -> torch.Tensor:
    if isinstance(v, torch.Tensor):
        return v.detach().to(device=dev, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.asarray(v, dtype=np.float64), device=dev).contiguous()


def accumulate_matrices(matrices):
    """transfer.py:115-137: matrices[-1] @ ... @ matrices[0]."""
    if len(matrices) == 0:
        raise IndexError("accumulate_matrices needs at least one matrix")
    total = matrices[-1]
    for tm in reversed(matrices[:-1]):
        total = total @ tm
    return total


def accumulate_matrices_cumulative(matrices) -> np.ndarray:
    """transfer.py:140-183, in the order the reference's loop builds them:
    result[0] = M[-1], result[k] = M[-1-k] @ result[k-1]."""
    a = _host_mats(matrices)
    if a.shape[0] == 0:
        raise IndexError("accumulate_matrices_cumulative needs at least one matrix")
    out = np.empty_like(a)
    N.check(N.lib().tg_transfer_cumulative(a.shape[0], a.ctypes.data, out.ctypes.data),
            "tg_transfer_cumulative")
    return out


def transfer_rays(ray_coords, transfer_matrices) -> torch.Tensor:
    """transfer.py:6-53: (N, 5) rays [x, y, dx, dy, 1] through each cumulative
    product of the (M, 5, 5) matrices -> (N, M, 5) float64 on the GPU."""
    mats = _host_mats(transfer_matrices)
    if mats.shape[0] == 0:
        raise IndexError("transfer_rays needs at least one transfer matrix")
    dev = _device()
    rays = _dev64(ray_coords, dev)
    if rays.ndim != 2 or rays.shape[1] != 5:
        raise ValueError("ray_coords must have shape (N, 5)")
    n, m = rays.shape[0], mats.shape[0]
    out = torch.empty((n, m, 5), dtype=torch.float64, device=dev)
    N.check(N.lib().tg_transfer_rays(n, rays.data_ptr(), m, mats.ctypes.data, out.data_ptr(),
                                     N.stream_ptr()), "tg_transfer_rays")
    return out


def transfer_rays_pt_src(input_pos_xy, input_slopes_xy, transfer_matrix) -> torch.Tensor:
    """transfer.py:56-112: rays from one point with the given slopes through a
    5x5 matrix -> (4, N) float64 rows x, y, dx, dy on the GPU."""
    x0, y0 = (float(v) for v in input_pos_xy)
    dev = _device()
    sx, sy = (_dev64(v, dev).reshape(-1) for v in input_slopes_xy)
    if sx.numel() != sy.numel():
        raise ValueError("slope arrays must have the same length")
    t = np.ascontiguousarray(np.asarray(
        transfer_matrix.detach().cpu().numpy() if isinstance(transfer_matrix, torch.Tensor) else transfer_matrix,
        dtype=np.float64))
    if t.shape != (5, 5):
        raise ValueError("transfer_matrix must be 5x5")
    n = sx.numel()
    out = torch.empty((4, n), dtype=torch.float64, device=dev)
    N.check(N.lib().tg_transfer_rays_pt_src(x0, y0, n, sx.data_ptr(), sy.data_ptr(), t.ctypes.data,
                                            out.data_ptr(), N.stream_ptr()), "tg_transfer_rays_pt_src")
    return out
