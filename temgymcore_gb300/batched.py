"""Many independent optical models in one persistent GPU launch.

``BatchedTrace(models, rays_per_model)`` packs every model into one device
plan (``tg_batch_plan``) and runs forward (+ adjoint of a squared-residual
loss when targets are given) over all of them in a single launch
(``tg_batch_run``), optionally captured as a CUDA graph.  Launch shape (tile
size, block size, rays per thread) is picked by a small autotuner that times
the candidates on the actual workload and caches the winner per workload
signature (host-side, lock-protected, optionally persisted as JSON).

The reference evaluates each model separately: ``run_to_end``
(run.py:85-116) and ``jax.value_and_grad`` of a loss over it.
``BatchedTrace.value_and_grad`` is that pair for every model at once: the
loss is the sum over rays that every aperture passes of the squared
detector-position residual, and the gradient is returned as per-step sums
(``grads`` maps them to named component parameters).
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading

import numpy as np
import torch

from . import _native as N
from .run import _check_model, _device, pack_model, param_gradient


class TgBatchInfo(C.Structure):
    _fields_ = [("plan_bytes", C.c_size_t), ("workspace_bytes", C.c_size_t), ("n_tiles", C.c_int32),
                ("total_steps", C.c_int32), ("total_rays", C.c_int64), ("max_steps", C.c_int32),
                ("max_moments", C.c_int32), ("n_models", C.c_int32), ("partial_doubles", C.c_int64),
                ("moment_doubles", C.c_int64), ("max_record_floats", C.c_int32)]


class TgBatchIO(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("dx", C.c_void_p), ("dy", C.c_void_p),
                ("out_x", C.c_void_p), ("out_y", C.c_void_p), ("out_dx", C.c_void_p),
                ("out_dy", C.c_void_p), ("out_pathlength", C.c_void_p), ("target_x", C.c_void_p),
                ("target_y", C.c_void_p), ("raw", C.c_void_p), ("out_alive", C.c_void_p),
                ("loss", C.c_void_p)]


N.register("tg_batch_plan", C.c_int, [C.c_int32, C.POINTER(N.TgModel), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_double), C.c_int32, C.c_void_p, C.c_size_t,
                                      C.POINTER(TgBatchInfo)])
N.register("tg_batch_run", C.c_int, [C.c_void_p, C.POINTER(TgBatchInfo), C.POINTER(TgBatchIO), C.c_int32,
                                     C.c_int32, C.c_void_p, C.c_size_t, C.c_void_p])

# (tile rays, block, rays per thread) candidates
CANDIDATES = [(2048, 256, 2), (4096, 256, 2), (4096, 128, 4), (8192, 256, 2), (16384, 256, 2),
              (4096, 256, 4), (4096, 512, 2), (8192, 256, 4), (2048, 256, 1),
              (8192, 512, 2), (16384, 512, 2), (16384, 512, 1)]


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
        self._vg = None

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

    def io(self, x, y, dx, dy, out, targets=None, raw=None, alive=None, loss=None) -> TgBatchIO:
        for t in (x, y, dx, dy):
            if t.dtype != torch.float32 or not t.is_cuda or t.numel() != self.total:
                raise ValueError("ray inputs must be float32 CUDA tensors of every model's rays")
        b = TgBatchIO()
        b.x, b.y, b.dx, b.dy = (t.data_ptr() for t in (x, y, dx, dy))
        b.out_x, b.out_y, b.out_dx, b.out_dy, b.out_pathlength = (
            None if t is None else t.data_ptr() for t in out)
        if targets is not None:
            b.target_x, b.target_y = targets[0].data_ptr(), targets[1].data_ptr()
            b.raw = raw.data_ptr()
        if alive is not None:
            if alive.dtype != torch.uint8 or alive.numel() != self.total:
                raise ValueError("alive must be a uint8 tensor of every model's rays")
            b.out_alive = alive.data_ptr()
        if loss is not None:
            if targets is None:
                raise ValueError("the loss needs targets")
            if loss.dtype != torch.float64 or loss.numel() != len(self.models):
                raise ValueError("loss must be a float64 tensor with one entry per model")
            b.loss = loss.data_ptr()
        return b

    def alloc_outputs(self):
        f = lambda: torch.empty(self.total, dtype=torch.float32, device=self.dev)  # noqa: E731
        return (f(), f(), f(), f(), torch.empty(self.total, dtype=torch.float64, device=self.dev))

    def alloc_raw(self):
        return torch.zeros((int(self.info.total_steps), 4), dtype=torch.float64, device=self.dev)

    def alloc_alive(self):
        """Per-ray mask: 1 where every aperture passes the ray."""
        return torch.empty(self.total, dtype=torch.uint8, device=self.dev)

    def alloc_loss(self):
        return torch.zeros(len(self.models), dtype=torch.float64, device=self.dev)

    def run(self, x, y, dx, dy, out, targets=None, raw=None, block=None, rays_per_thread=None,
            alive=None, loss=None):
        io = self.io(x, y, dx, dy, out, targets, raw, alive, loss)
        st = N.lib().tg_batch_run(self.plan.data_ptr(), C.byref(self.info), C.byref(io),
                                  block or self.block, rays_per_thread or self.rpt,
                                  self.ws.data_ptr() + self.ws_off, self.ws.numel() - self.ws_off,
                                  N.stream_ptr())
        N.check(st, "tg_batch_run")

    def signature(self) -> str:
        return f"m{len(self.models)}-r{self.total}-s{int(self.info.total_steps)}"

    def autotune(self, x, y, dx, dy, out, targets=None, raw=None, reps=5, alive=None, loss=None):
        """Time each candidate launch shape on this workload; keep the fastest."""
        key = self.signature() + ("-adj" if targets is not None else "-fwd") + ("-mask" if alive is not None else "")
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
            self.run(x, y, dx, dy, out, targets, raw, block, rpt, alive=alive, loss=loss)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(reps):
                self.run(x, y, dx, dy, out, targets, raw, block, rpt, alive=alive, loss=loss)
            b.record()
            torch.cuda.synchronize()
            results.append((a.elapsed_time(b) / reps, tile, block, rpt))
        best = min(results)
        _, tile, self.block, self.rpt = best
        if tile != self.tile_rays:
            self._build(tile)
        TUNE_CACHE.put(key, (tile, self.block, self.rpt))
        return (tile, self.block, self.rpt), results

    def capture(self, x, y, dx, dy, out, targets=None, raw=None, alive=None, loss=None):
        """Capture one batched launch (forward [+ adjoint]) as a CUDA graph."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(x, y, dx, dy, out, targets, raw, alive=alive, loss=loss)
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(x, y, dx, dy, out, targets, raw, alive=alive, loss=loss)
        self.graph = g
        return g

    def value_and_grad(self, x, y, dx, dy, tx, ty, sync=True):
        """Loss and gradient of every model in one launch: the batched form of
        ``jax.value_and_grad`` over ``run_to_end`` (run.py:85-116) with
        loss_m = sum over model m's alive rays of (x_out - tx)^2 + (y_out - ty)^2.

        Inputs are float32 tensors of every model's rays (concatenated in model
        order), on the host or on the device.  Host inputs are copied in on
        the current stream and the results come back to pinned host memory;
        with ``sync=False`` the call returns without waiting, and the host
        results are valid once the current stream has synchronised (the next
        call reuses the same buffers).  Returns (loss [n_models], raw
        [total_steps, 4]) float64; ``grads(raw, m)`` names model m's
        parameter gradients.  The forward outputs stay on the device in
        ``self.last_outputs`` (x, y, dx, dy, pathlength, alive)."""
        host = not x.is_cuda
        if self._vg is None:
            out = self.alloc_outputs()
            dev_in = torch.empty((6, self.total), dtype=torch.float32, device=self.dev)
            self._vg = {"out": out, "alive": self.alloc_alive(), "raw": self.alloc_raw(),
                        "loss": self.alloc_loss(), "in": dev_in,
                        "h_loss": torch.empty(len(self.models), dtype=torch.float64).pin_memory(),
                        "h_raw": torch.empty((int(self.info.total_steps), 4),
                                             dtype=torch.float64).pin_memory()}
        v = self._vg
        if host:
            for i, t in enumerate((x, y, dx, dy, tx, ty)):
                v["in"][i].copy_(t.reshape(-1), non_blocking=True)
            args = tuple(v["in"][i] for i in range(6))
        else:
            args = (x, y, dx, dy, tx, ty)
        self.run(*args[:4], v["out"], (args[4], args[5]), v["raw"], alive=v["alive"], loss=v["loss"])
        self.last_outputs = (*v["out"], v["alive"])
        if not host:
            return v["loss"], v["raw"]
        v["h_loss"].copy_(v["loss"], non_blocking=True)
        v["h_raw"].copy_(v["raw"], non_blocking=True)
        if sync:
            torch.cuda.current_stream().synchronize()
        return v["h_loss"], v["h_raw"]

    def grads(self, raw, m: int, paths=("z", "focal_length", "def_x", "def_y")):
        """Model m's gradient by component: a list (one dict per component) of
        d loss / d field for the fields of ``paths`` that the component has."""
        comps = self.models[m]
        r = torch.as_tensor(self.model_raw(raw, m), dtype=torch.float64)
        out = []
        for i, c in enumerate(comps):
            d = {}
            for p in paths:
                if p == "z" or hasattr(c, p):
                    d[p] = float(param_gradient(comps, i, p, r))
            out.append(d)
        return out

    def model_raw(self, raw: torch.Tensor, m: int) -> torch.Tensor:
        """Per-step sums of model m (rows 2*len(model))."""
        return raw[int(self.step_offsets[m]):int(self.step_offsets[m + 1])]
