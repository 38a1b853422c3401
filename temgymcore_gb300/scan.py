"""4D-STEM batch: per-scan-position detector images in one launch.

The reference produces a shadow image per scan position by rebuilding the
model with that position's Scanner/Descanner and calling ``run_to_end`` then
``Detector.into_image`` (run.py:85-116, grid.py:231-280) - one Python call per
position.  ``scan_images`` runs every position in one persistent kernel: each
Scanner and Descanner in the model takes the probe's scan position (their
own ``scan_pos_*`` fields are ignored); tilts and descan errors are kept.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np
import torch

from . import _native as N
from .components import Descanner, Detector, Grid, ScanGrid, Scanner
from .ray import Ray, as_f32, as_f64_or_scalar
from .run import _check_model, _device, _rays_struct

N.register("tg_scan_hist", C.c_int, [C.POINTER(N.TgModel), C.POINTER(N.TgRays), C.c_void_p,
                                     C.POINTER(N.TgGrid), C.c_void_p, C.c_void_p, C.c_void_p])


class TgScan(C.Structure):
    _fields_ = [("n_probes", C.c_int32), ("cols", C.c_int32), ("t", C.c_double * 6),
                ("positions", C.c_void_p)]


def pack_scan_model(model):
    comps = _check_model(model)
    arr = (N.TgComponent * max(1, len(comps)))()
    for i, c in enumerate(comps):
        c._pack(arr[i])
        if isinstance(c, (Scanner, Descanner)):
            arr[i].flags = N.FLAG_PER_PROBE
    m = N.TgModel()
    m.n_components = len(comps)
    m.components = C.cast(arr, C.POINTER(N.TgComponent))
    return m, arr


def scan_struct(scan_grid: ScanGrid | None, positions=None, n_probes=None):
    s = TgScan()
    keep = None
    if positions is not None:
        pos = torch.as_tensor(positions, dtype=torch.float64, device=_device()).reshape(-1, 2).contiguous()
        s.n_probes = pos.shape[0]
        s.cols = 1
        s.positions = pos.data_ptr()
        keep = pos
    else:
        t = scan_grid.pixels_to_metres_mat
        s.n_probes = int(scan_grid.shape[0]) * int(scan_grid.shape[1]) if n_probes is None else n_probes
        s.cols = int(scan_grid.shape[1])
        for i, v in enumerate((t[0, 0], t[0, 1], t[0, 2], t[1, 0], t[1, 1], t[1, 2])):
            s.t[i] = float(v)
        s.positions = None
    return s, keep


def scan_positions(scan_grid: ScanGrid) -> np.ndarray:
    """(n_probes, 2) float64 (x, y) scan positions in probe order (row-major)."""
    h, w = int(scan_grid.shape[0]), int(scan_grid.shape[1])
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    x, y = scan_grid.pixels_to_metres((yy.ravel(), xx.ravel()))
    return np.stack([x, y], axis=-1)


def scan_shard(scan_grid: ScanGrid, rank: int, world: int):
    """Probe range and positions of one rank when a scan is split over
    ``world`` GPUs: contiguous row-major probe ranges whose sizes differ by at
    most one.  The probes are independent, so the ranks need no exchange; the
    images of rank r are probes [start, stop) of the full scan.
    Returns (start, stop, positions (stop - start, 2))."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must satisfy 0 <= rank < world")
    n = int(scan_grid.shape[0]) * int(scan_grid.shape[1])
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop, scan_positions(scan_grid)[start:stop]


def scan_images(ray: Ray, model, scan_grid: ScanGrid | None = None, detector: Grid | None = None,
                positions=None, out: torch.Tensor | None = None, return_xy: bool = False):
    """Dense int32 images (n_probes, H, W): the bundle ``ray`` traced through
    ``model`` at every scan position of ``scan_grid`` (row-major probe order)
    or of ``positions`` ((n, 2) x, y metres), binned on ``detector``
    (default: the model's last component).  With ``return_xy`` also returns
    the per-probe detector coordinates (n_probes, 2, n_rays) float32.
    ``out`` may be a pinned host tensor: the kernel then writes the images
    straight across the host link (no separate copy)."""
    comps = _check_model(model)
    if scan_grid is None and positions is None:
        found = [c for c in comps if isinstance(c, ScanGrid)]
        if not found:
            raise ValueError("scan_images needs a ScanGrid (in the model or as scan_grid=) or positions=")
        scan_grid = found[0]
    if detector is None:
        detector = comps[-1]
    if not isinstance(detector, Grid):
        raise ValueError("the detector must be a Detector/ScanGrid")
    dev = _device()
    n = ray.size
    x, y = as_f32(ray.x, n, dev), as_f32(ray.y, n, dev)
    dx, dy = as_f32(ray.dx, n, dev), as_f32(ray.dy, n, dev)
    zt, zs = as_f64_or_scalar(ray.z, n, dev)
    if zt is not None:
        raise NotImplementedError("scan_images needs one source plane (uniform z)")
    pt, ps = as_f64_or_scalar(ray.pathlength, n, dev)
    bundle = _rays_struct(n, x, y, dx, dy, None, zs, pt, ps)
    s, keep_pos = scan_struct(scan_grid, positions)
    h, w = int(detector.shape[0]), int(detector.shape[1])
    if out is None:
        out = torch.empty((s.n_probes, h, w), dtype=torch.int32, device=dev)
    if tuple(out.shape) != (s.n_probes, h, w) or out.dtype != torch.int32 or not out.is_contiguous():
        raise ValueError("out must be a contiguous int32 tensor (n_probes, H, W)")
    if not out.is_cuda and not out.is_pinned():
        raise ValueError("out must be a CUDA tensor or a pinned host tensor")
    xy = torch.empty((s.n_probes, 2, n), dtype=torch.float32, device=dev) if return_xy else None
    m, keep = pack_scan_model(comps)
    g = detector._tg_grid()
    N.check(N.lib().tg_scan_hist(C.byref(m), C.byref(bundle), C.byref(s), C.byref(g), N.ptr(out),
                                 N.ptr(xy), N.stream_ptr()), "tg_scan_hist")
    del keep, keep_pos
    return (out, xy) if return_xy else out


def probe_model(model, spx: float, spy: float):
    """The model at one scan position (what the reference rebuilds per probe)."""
    out = []
    for c in model:
        if isinstance(c, (Scanner, Descanner)):
            c = dataclasses.replace(c, scan_pos_x=spx, scan_pos_y=spy)
        out.append(c)
    return out
