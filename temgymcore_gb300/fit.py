"""Device-resident 4D-STEM calibration fit (descan error, camera length, scan
rotation, scan step, focal length, defocus).

The reference fits these by differentiating a loss over ``run_to_end`` with
``jax.grad`` (README.md:113-160) and stepping an optimiser on the host.  Here
the parameters stay in device memory: one fused forward+adjoint kernel
produces the loss and all 21 gradients (``tg_stem_fit_loss_grad``), and a
whole optimisation step (``tg_stem_fit_step``: the same pass, with the Adam
update applied by the reduction's last block) is two launches, captured once
in a CUDA graph and replayed for every step.  ``tg_adam_step`` alone updates
from any gradient.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .components import DescanError, Detector, Lens, ScanGrid, Scanner, Descanner, PointSource
from .ray import Ray, as_f32
from .run import _device


class TgStemFit(C.Structure):
    _fields_ = [("n_rays", C.c_int32), ("rows", C.c_int32), ("cols", C.c_int32),
                ("x", C.c_void_p), ("y", C.c_void_p), ("dx", C.c_void_p), ("dy", C.c_void_p),
                ("target_x", C.c_void_p), ("target_y", C.c_void_p), ("lens_gap", C.c_double)]


N.register("tg_stem_fit_forward", C.c_int, [C.POINTER(TgStemFit), C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p])
N.register("tg_stem_fit_workspace", C.c_size_t, [C.c_int32])
N.register("tg_stem_fit_loss_grad", C.c_int, [C.POINTER(TgStemFit), C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_size_t, C.c_void_p])
N.register("tg_adam_step", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.c_void_p])
N.register("tg_stem_fit_step", C.c_int, [C.POINTER(TgStemFit), C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                         C.c_void_p])

PARAM_NAMES = (["focal_length", "defocus", "camera_length", "scan_rotation", "scan_step"]
               + [f"M[{r}][{c}]" for r in range(4) for c in range(4)])


def theta_from(f, defocus, camera_length, scan_rotation, scan_step, descan):
    """float64 parameter vector in the kernel's order."""
    return np.concatenate([[f, defocus, camera_length, scan_rotation, scan_step],
                           np.asarray(descan, dtype=np.float64).reshape(16)])


class StemFit:
    """Loss/gradient/Adam on the device for one ray bundle and a rows x cols scan."""

    def __init__(self, bundle: Ray, rows: int, cols: int, lens_gap: float, theta, targets=None):
        self.dev = _device()
        n = bundle.size
        self.n, self.rows, self.cols, self.gap = n, int(rows), int(cols), float(lens_gap)
        self.x, self.y = as_f32(bundle.x, n, self.dev), as_f32(bundle.y, n, self.dev)
        self.dx, self.dy = as_f32(bundle.dx, n, self.dev), as_f32(bundle.dy, n, self.dev)
        self.theta = torch.as_tensor(np.asarray(theta, np.float64), device=self.dev).clone()
        self.n_probes = self.rows * self.cols
        self.tx = torch.zeros((self.n_probes, n), dtype=torch.float32, device=self.dev)
        self.ty = torch.zeros_like(self.tx)
        if targets is not None:
            self.tx.copy_(targets[0])
            self.ty.copy_(targets[1])
        self.out = torch.zeros(22, dtype=torch.float64, device=self.dev)
        nbytes = N.lib().tg_stem_fit_workspace(self.n_probes)
        self.ws = torch.empty(max(8, nbytes), dtype=torch.uint8, device=self.dev)
        self.m = torch.zeros(21, dtype=torch.float64, device=self.dev)
        self.v = torch.zeros_like(self.m)
        self.t = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.scale = torch.ones(21, dtype=torch.float64, device=self.dev)
        self.mask = torch.ones(21, dtype=torch.uint8, device=self.dev)
        self.graph = None

    def _cfg(self) -> TgStemFit:
        c = TgStemFit()
        c.n_rays, c.rows, c.cols = self.n, self.rows, self.cols
        c.x, c.y, c.dx, c.dy = (t.data_ptr() for t in (self.x, self.y, self.dx, self.dy))
        c.target_x, c.target_y = self.tx.data_ptr(), self.ty.data_ptr()
        c.lens_gap = self.gap
        return c

    def forward(self, theta=None):
        """Detector (x, y) of every (probe, ray): two (n_probes, n) float32 tensors."""
        th = self.theta if theta is None else torch.as_tensor(theta, dtype=torch.float64, device=self.dev)
        ox = torch.empty((self.n_probes, self.n), dtype=torch.float32, device=self.dev)
        oy = torch.empty_like(ox)
        N.check(N.lib().tg_stem_fit_forward(C.byref(self._cfg()), th.data_ptr(), ox.data_ptr(),
                                            oy.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
                                            N.stream_ptr()), "tg_stem_fit_forward")
        return ox, oy

    def set_targets(self, theta_true):
        ox, oy = self.forward(theta_true)
        self.tx.copy_(ox)
        self.ty.copy_(oy)

    def loss_grad(self):
        """out[0] = loss, out[1:] = gradient (device float64 [22])."""
        N.check(N.lib().tg_stem_fit_loss_grad(C.byref(self._cfg()), self.theta.data_ptr(),
                                              self.out.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
                                              N.stream_ptr()), "tg_stem_fit_loss_grad")
        return self.out

    def adam(self, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        N.check(N.lib().tg_adam_step(self.theta.data_ptr(), self.out.data_ptr() + 8, self.m.data_ptr(),
                                     self.v.data_ptr(), self.t.data_ptr(), 21, lr, betas[0], betas[1],
                                     eps, self.scale.data_ptr(), self.mask.data_ptr(),
                                     N.stream_ptr()), "tg_adam_step")

    def step(self, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        """loss_grad + adam in two launches (out holds the loss and gradient
        at the parameters before the update)."""
        N.check(N.lib().tg_stem_fit_step(C.byref(self._cfg()), self.theta.data_ptr(), self.out.data_ptr(),
                                         self.m.data_ptr(), self.v.data_ptr(), self.t.data_ptr(), lr,
                                         betas[0], betas[1], eps, self.scale.data_ptr(),
                                         self.mask.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
                                         N.stream_ptr()), "tg_stem_fit_step")

    def capture(self, lr=1e-3):
        """Capture one loss/gradient/Adam step as a CUDA graph."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.loss_grad()  # warm-up outside capture
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(lr)
        self.graph = g
        return g

    def fit(self, steps=200, lr=1e-3, use_graph=True):
        """Run ``steps`` Adam steps; returns the loss before each step (device)."""
        hist = torch.empty(steps, dtype=torch.float64, device=self.dev)
        if use_graph:
            if self.graph is None:
                self.capture(lr)
            for i in range(steps):
                self.graph.replay()
                hist[i] = self.out[0]
        else:
            for i in range(steps):
                self.step(lr)
                hist[i] = self.out[0]
        return hist

    def identifiable(self, theta=None) -> np.ndarray:
        """``identifiable_combinations`` of theta (default: the current
        parameters) for this scan and lens gap."""
        th = self.theta if theta is None else theta
        th = th.detach().cpu().numpy() if isinstance(th, torch.Tensor) else th
        return identifiable_combinations(th, self.gap, self.rows, self.cols)

    def model_at(self, theta, spx=0.0, spy=0.0):
        """The equivalent component model at one scan position (reference form)."""
        th = np.asarray(theta.detach().cpu() if isinstance(theta, torch.Tensor) else theta, np.float64)
        f, dfc, cl, rot, step = th[:5]
        err = DescanError.from_matrix4(th[5:].reshape(4, 4))
        return [PointSource(z=0.0),
                ScanGrid(z=dfc, pixel_size=(step, step), shape=(self.rows, self.cols), rotation=rot),
                Scanner(z=dfc, scan_pos_x=spx, scan_pos_y=spy),
                Descanner(z=dfc, scan_pos_x=spx, scan_pos_y=spy, descan_error=err),
                Lens(z=dfc + self.gap, focal_length=f),
                Detector(z=dfc + cl, pixel_size=(1e-5, 1e-5), shape=(256, 256))]


def identifiable_combinations(theta, lens_gap: float, rows: int, cols: int) -> np.ndarray:
    """The six combinations of the 21 parameters that the detector positions
    determine (parameter vectors with equal combinations give the same loss).
    From the scan plane the lens section maps (x, dx) to x_det = A x + B dx,
    A = 1 - (cl - gap) / f, B = gap + (cl - gap)(1 - gap / f); a bundle ray
    (x0, dx0) reaches the scan plane at x0 + defocus dx0; the scan adds the
    descan matrix's position rows to x and its slope rows to dx, times the
    scan position S (row, col) (S: the ScanGrid's pixel -> metre map, which
    holds the rotation and the step).  So the detector sees only
      a = A, b = A defocus + B   (the bundle's position and slope gains),
      K = (A M[0:2, 0:2] + B M[2:4, 0:2]) S   (2 x 2: scan pixel -> detector),
    returned as [a, b, K00, K01, K10, K11]; the descan tilt columns
    M[:, 2:4] do not enter at all (the scan tilt is 0)."""
    th = np.asarray(theta, np.float64)
    f, dfc, cl, rot, step = th[:5]
    M = th[5:].reshape(4, 4)
    g = float(lens_gap)
    A = 1.0 - (cl - g) / f
    B = g + (cl - g) * (1.0 - g / f)
    t = ScanGrid(z=dfc, pixel_size=(step, step), shape=(int(rows), int(cols)),
                 rotation=rot).pixels_to_metres_mat
    S = np.array([[t[1, 0], t[1, 1]], [t[0, 0], t[0, 1]]])  # (x, y) per (row, col)
    K = (A * M[0:2, 0:2] + B * M[2:4, 0:2]) @ S
    return np.concatenate([[A, A * dfc + B], K.reshape(4)])
