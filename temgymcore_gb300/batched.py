"""Many independent optical models in one persistent GPU launch.

``BatchedTrace(models, rays_per_model)`` packs every model into one device
plan (``tg_batch_plan``) and runs forward (+ adjoint of a squared-residual
loss when targets are given) over all of them in a single launch
(``tg_batch_run``), optionally captured as a CUDA graph.  Launch shape (tile
size, block size, rays per thread) is picked by a small autotuner that times
the candidates on the actual workload and caches the winner per workload
signature (host-side, lock-protected, optionally persisted as JSON).
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading

import numpy as np
import torch

from . import _native as N
from .run import _check_model, _device, pack_model


class TgBatchInfo(C.Structure):
    _fields_ = [("plan_bytes", C.c_size_t), ("workspace_bytes", C.c_size_t), ("n_tiles", C.c_int32),
                ("total_steps", C.c_int32), ("total_rays", C.c_int64), ("max_steps", C.c_int32),
                ("max_moments", C.c_int32), ("n_models", C.c_int32), ("partial_doubles", C.c_int64),
                ("moment_doubles", C.c_int64)]


class TgBatchIO(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("dx", C.c_void_p), ("dy", C.c_void_p),
                ("out_x", C.c_void_p), ("out_y", C.c_void_p), ("out_dx", C.c_void_p),
                ("out_dy", C.c_void_p), ("out_pathlength", C.c_void_p), ("target_x", C.c_void_p),
                ("target_y", C.c_void_p), ("raw", C.c_void_p)]


N.register("tg_batch_plan", C.c_int, [C.c_int32, C.POINTER(N.TgModel), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_double), C.c_int32, C.c_void_p, C.c_size_t,
                                      C.POINTER(TgBatchInfo)])
N.register("tg_batch_run", C.c_int, [C.c_void_p, C.POINTER(TgBatchInfo), C.POINTER(TgBatchIO), C.c_int32,
                                     C.c_int32, C.c_void_p, C.c_size_t, C.c_void_p])

# (tile rays, block, rays per thread) candidates
CANDIDATES = [(2048, 256, 2), (4096, 256, 2), (4096, 128, 4), (8192, 256, 2), (16384, 256, 2),
              (4096, 256, 4), (4096, 512, 2), (8192, 256, 4), (2048, 256, 1)]


class _TuneCache:
    def __init__(self):
        self.lock = threading.Lock()
        self.mem: dict[str, list] = {}
        self.path = os.environ.get("TEMGYM_GB300_TUNE_CACHE")
        if self.path and os.path.exists(self.path):
            try:
                with open(self.path) as fh:
                    self.mem.update(json.load(fh))
            except Exception:
                pass

    def get(self, key):
        with self.lock:
            return self.mem.get(key)

    def put(self, key, val):
        with self.lock:
            self.mem[key] = list(val)
            if self.path:
                tmp = self.path + ".tmp"
                with open(tmp, "w") as fh:
                    json.dump(self.mem, fh)
                os.replace(tmp, self.path)


TUNE_CACHE = _TuneCache()


class BatchedTrace:
    """models: list of component lists; n_rays: rays per model.  Ray arrays are
    concatenated in model order (float32 device tensors of sum(n_rays))."""

    def __init__(self, models, n_rays, z_in=None, tile_rays=2048):
        self.dev = _device()
        self.models = [_check_model(m) for m in models]
        self.n_rays = np.asarray(n_rays, dtype=np.int64)
        self.z_in = None if z_in is None else np.asarray(z_in, dtype=np.float64)
        self.offsets = np.concatenate([[0], np.cumsum(self.n_rays)])
        self.total = int(self.offsets[-1])
        self.step_offsets = np.concatenate([[0], np.cumsum([2 * len(m) for m in self.models])])
        self._packed = [pack_model(m) for m in self.models]
        self._build(tile_rays)
        self.block, self.rpt = 256, 2
        self.graph = None

    def _build(self, tile_rays):
        arr = (N.TgModel * max(1, len(self.models)))()
        for i, (m, _) in enumerate(self._packed):
            arr[i] = m
        self._arr = arr
        cnt = (C.c_int64 * max(1, len(self.models)))(*self.n_rays.tolist())
        zin = None if self.z_in is None else (C.c_double * len(self.models))(*self.z_in.tolist())
        info = TgBatchInfo()
        N.check(N.lib().tg_batch_plan(len(self.models), arr, cnt, zin, tile_rays, None, 0, C.byref(info)),
                "tg_batch_plan")
        host = np.zeros(info.plan_bytes, dtype=np.uint8)
        N.check(N.lib().tg_batch_plan(len(self.models), arr, cnt, zin, tile_rays, host.ctypes.data,
                                      host.nbytes, C.byref(info)), "tg_batch_plan")
        self.info = info
        self.tile_rays = tile_rays
        self.plan = torch.as_tensor(host, device=self.dev)
        self.ws = torch.empty(info.workspace_bytes + 256, dtype=torch.uint8, device=self.dev)
        self.ws_off = (-self.ws.data_ptr()) % 256

    def io(self, x, y, dx, dy, out, targets=None, raw=None) -> TgBatchIO:
        b = TgBatchIO()
        b.x, b.y, b.dx, b.dy = (t.data_ptr() for t in (x, y, dx, dy))
        b.out_x, b.out_y, b.out_dx, b.out_dy, b.out_pathlength = (
            None if t is None else t.data_ptr() for t in out)
        if targets is not None:
            b.target_x, b.target_y = targets[0].data_ptr(), targets[1].data_ptr()
            b.raw = raw.data_ptr()
        return b

    def alloc_outputs(self):
        f = lambda: torch.empty(self.total, dtype=torch.float32, device=self.dev)  # noqa: E731
        return (f(), f(), f(), f(), torch.empty(self.total, dtype=torch.float64, device=self.dev))

    def alloc_raw(self):
        return torch.zeros((int(self.info.total_steps), 4), dtype=torch.float64, device=self.dev)

    def run(self, x, y, dx, dy, out, targets=None, raw=None, block=None, rays_per_thread=None):
        io = self.io(x, y, dx, dy, out, targets, raw)
        st = N.lib().tg_batch_run(self.plan.data_ptr(), C.byref(self.info), C.byref(io),
                                  block or self.block, rays_per_thread or self.rpt,
                                  self.ws.data_ptr() + self.ws_off, self.ws.numel() - self.ws_off,
                                  N.stream_ptr())
        N.check(st, "tg_batch_run")

    def signature(self) -> str:
        return f"m{len(self.models)}-r{self.total}-s{int(self.info.total_steps)}"

    def autotune(self, x, y, dx, dy, out, targets=None, raw=None, reps=5):
        """Time each candidate launch shape on this workload; keep the fastest."""
        key = self.signature() + ("-adj" if targets is not None else "-fwd")
        hit = TUNE_CACHE.get(key)
        if hit:
            tile, self.block, self.rpt = hit
            if tile != self.tile_rays:
                self._build(tile)
            return hit, None
        results = []
        for tile, block, rpt in CANDIDATES:
            if tile != self.tile_rays:
                self._build(tile)
            self.run(x, y, dx, dy, out, targets, raw, block, rpt)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(reps):
                self.run(x, y, dx, dy, out, targets, raw, block, rpt)
            b.record()
            torch.cuda.synchronize()
            results.append((a.elapsed_time(b) / reps, tile, block, rpt))
        best = min(results)
        _, tile, self.block, self.rpt = best
        if tile != self.tile_rays:
            self._build(tile)
        TUNE_CACHE.put(key, (tile, self.block, self.rpt))
        return (tile, self.block, self.rpt), results

    def capture(self, x, y, dx, dy, out, targets=None, raw=None):
        """Capture one batched launch (forward [+ adjoint]) as a CUDA graph."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(x, y, dx, dy, out, targets, raw)
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(x, y, dx, dy, out, targets, raw)
        self.graph = g
        return g

    def model_raw(self, raw: torch.Tensor, m: int) -> torch.Tensor:
        """Per-step sums of model m (rows 2*len(model))."""
        return raw[int(self.step_offsets[m]):int(self.step_offsets[m + 1])]
