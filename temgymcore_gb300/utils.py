"""Helpers of temgym_core.utils on the path (utils.py:7-43, 83-114, 285-294).

``custom_jacobian_matrix`` turns a Ray-of-Rays Jacobian into the 5x5
homogeneous matrix; ``inplace_sum`` is the detector accumulation of
``Grid.into_image`` on the GPU; ``make_aperture`` is the image-plane disc mask
used by the reference's tests.  Ray sources' ``concentric_rings`` /
``random_coords`` and ``fibonacci_spiral`` are re-exported.
"""
from __future__ import annotations

import numpy as np
import torch

from .gaussian import fibonacci_spiral  # noqa: F401
from .sources import concentric_rings, random_coords  # noqa: F401

_ROWS = ("x", "y", "dx", "dy", "_one")


def _val(v):
    if isinstance(v, torch.Tensor):
        return v.detach().cpu().numpy().astype(np.float64)
    return np.asarray(v, dtype=np.float64)


def custom_jacobian_matrix(ray_jac) -> np.ndarray:
    """utils.py:7-43: rows and columns [x, y, dx, dy, _one] of a Ray-of-Rays
    Jacobian (``jacobian_transform``, ``run_with_grads``) as a float64 array
    (..., 5, 5)."""
    rows = []
    for r in _ROWS:
        out_r = getattr(ray_jac, r)
        rows.append(np.stack(np.broadcast_arrays(*[_val(getattr(out_r, c)) for c in _ROWS]), axis=-1))
    return np.stack(np.broadcast_arrays(*rows), axis=-2)


def make_aperture(X, Y, aperture_ratio: float = 0.1):
    """utils.py:285-294: boolean disc of radius aperture_ratio * max|X| on the
    coordinate grids X, Y (an image-plane mask); NumPy in, NumPy out, and
    torch tensors stay torch tensors on their device."""
    if isinstance(X, torch.Tensor) or isinstance(Y, torch.Tensor):
        Xt, Yt = torch.as_tensor(X), torch.as_tensor(Y)
        radius = aperture_ratio * Xt.abs().max()
        return (Xt ** 2 + Yt ** 2) < radius ** 2
    X, Y = np.asarray(X), np.asarray(Y)
    radius = np.max(np.abs(X)) * aperture_ratio
    return X ** 2 + Y ** 2 < radius ** 2


_DTYPES = {torch.int32: 0, torch.int64: 1, torch.float32: 2, torch.float64: 3}


def inplace_sum(px_y, px_x, mask, frame, buffer):
    """utils.py:83-114 on the GPU: buffer[py, px] += frame[i] for every i with
    mask[i] and (py, px) inside the buffer.  ``buffer`` (2-D, int32 / int64 /
    float32 / float64) is updated in place: a contiguous CUDA tensor directly,
    a NumPy array by a copy to the device and back.  ``mask`` / ``frame`` may
    be None (all hits / add 1).  Integer buffers are exact; float buffers
    match the serial sum to its rounding (the adds land in any order)."""
    import ctypes as C

    from . import _native as N
    from .run import _device
    dev = _device()
    host = None
    if isinstance(buffer, torch.Tensor):
        if not (buffer.is_cuda and buffer.is_contiguous()):
            raise ValueError("buffer must be a contiguous CUDA tensor (or a NumPy array)")
        buf = buffer
    else:
        host = buffer
        buf = torch.as_tensor(np.ascontiguousarray(buffer), device=dev)
    if buf.dim() != 2 or buf.dtype not in _DTYPES:
        raise TypeError("buffer must be 2-D int32, int64, float32 or float64")
    h, w = buf.shape
    idx = lambda v: torch.as_tensor(v, device=dev).to(torch.int64).reshape(-1).contiguous()  # noqa: E731
    py, px = idx(px_y), idx(px_x)
    n = py.numel()
    if px.numel() != n:
        raise ValueError("px_y and px_x differ in length")
    m = None if mask is None else torch.as_tensor(mask, device=dev).reshape(-1).to(torch.uint8).contiguous()
    f = None if frame is None else torch.as_tensor(frame, device=dev).reshape(-1).to(buf.dtype).contiguous()
    if (m is not None and m.numel() != n) or (f is not None and f.numel() != n):
        raise ValueError("mask / frame must have one entry per hit")
    N.register("tg_inplace_sum", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                           C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                           C.c_void_p])
    N.check(N.lib().tg_inplace_sum(n, py.data_ptr(), px.data_ptr(), 1, N.ptr(m), N.ptr(f),
                                   _DTYPES[buf.dtype], h, w, buf.data_ptr(), N.stream_ptr()),
            "tg_inplace_sum")
    if host is not None:
        host[...] = buf.cpu().numpy()
    return None


def try_ravel(val):
    """utils.py:207-222: val.ravel() where it exists (torch: reshape(-1)),
    else val."""
    if isinstance(val, torch.Tensor):
        return val.reshape(-1)
    try:
        return val.ravel()
    except AttributeError:
        return val


def try_reshape(val, maybe_has_shape):
    """utils.py:225-242: val reshaped to maybe_has_shape.shape where both
    allow it, else val."""
    try:
        return val.reshape(tuple(maybe_has_shape.shape))
    except AttributeError:
        return val


def zero_phase(u, idx_x, idx_y):
    """utils.py:276-280: multiply the field u in place by the phase that makes
    u[idx_x, idx_y] real and non-negative; returns u."""
    c = u[idx_x, idx_y]
    if isinstance(u, torch.Tensor):
        u *= torch.exp(-1j * torch.angle(c))
        return u
    u *= np.exp(1j * (0 - np.angle(c)))
    return u


def multi_cumsum_inplace(values, partitions, start):
    """utils.py:47-80: running sums over ``values`` (1-D, modified in place)
    that restart at ``start`` once a partition's length has been counted.
    The count starts after the first element of each partition, so each
    restart lands one index after the partition boundary - the layout the
    reference's concentric_rings relies on, reproduced here as is.  Host
    helper; the ray sources run the same recurrence on the GPU."""
    parts = [int(p) for p in np.asarray(partitions).reshape(-1)]
    if values.size == 0:
        return None
    part, length, count = 0, parts[0], 0
    values[0] = start
    for i in range(1, values.size):
        if count == length:
            count = 0
            part += 1
            length = parts[part]
            values[i] = start
        else:
            values[i] += values[i - 1]
            count += 1
    return None


def FresnelPropagator(u1, L, wavelength, z, xp=np):  # noqa: N802 - the reference's name
    """utils.py:245-262: Fresnel propagation of the square field u1 (side L)
    over z by the transfer-function method, U2 = IFFT(H FFT(u1)) with
    H = exp(-i pi wavelength z (fx^2 + fy^2)).  torch tensors (or
    xp=torch) run with torch.fft on their device; anything else with NumPy."""
    if isinstance(u1, torch.Tensor) or xp is torch:
        t = torch.as_tensor(u1)
        m, n = t.shape
        d = L / m
        fx = torch.fft.fftfreq(n, d=d, device=t.device, dtype=torch.float64)
        fy = torch.fft.fftfreq(m, d=d, device=t.device, dtype=torch.float64)
        FY, FX = torch.meshgrid(fy, fx, indexing="ij")
        H = torch.exp(-1j * torch.pi * wavelength * z * (FX ** 2 + FY ** 2))
        return torch.fft.ifft2(H * torch.fft.fft2(t))
    m, n = u1.shape
    d = L / m
    FX, FY = np.meshgrid(np.fft.fftfreq(n, d=d), np.fft.fftfreq(m, d=d))
    return np.fft.ifft2(np.exp(-1j * np.pi * wavelength * z * (FX ** 2 + FY ** 2)) * np.fft.fft2(u1))


def fresnel_lens_imaging_solution(E0, Y, X, ps, lambda0, z1, f, z2):  # noqa: N803
    """utils.py:265-272: E0 propagated z1, through a thin lens of focal length
    f (phase exp(-i k (X^2 + Y^2) / 2f)), then z2; square grid of pixel ps."""
    k = 2 * np.pi / lambda0
    side = E0.shape[0] * ps
    E = FresnelPropagator(E0, side, lambda0, z1)
    lib = torch if isinstance(E, torch.Tensor) else np
    E = E * lib.exp((-1j * k) / (2 * f) * (X ** 2 + Y ** 2))
    return FresnelPropagator(E, side, lambda0, z2)
