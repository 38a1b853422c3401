"""Gaussian-beamlet detector field (drop-in for gaussian.py:225-369).

``make_gaussian_image(gaussian_rays, model)`` returns the complex64 detector
field (H, W) on the GPU.  The per-beam float64 preparation (ABCD of each
central ray, Q2^-1, prefactor, exact k*pathlength reduction) and the sum over
beams x pixels run in the C-ABI kernels of ``csrc/field.cu`` and
``csrc/field_gemm.cu``:

  method="separable"  diagonal Q2 on an unrotated grid: split-BF16 complex
                      GEMM on the tcgen05 tensor cores;
  method="direct"     any Q2 (astigmatic beams): exact fixed-point phase,
                      float32 geometric recurrence along each pixel strip;
  method="fp64"       every (beam, pixel) term in float64 (comparator);
  method="auto"       "separable" when every beam qualifies, else "direct".

``evaluate_gaussian_input_image(gaussian_rays, grid)`` (gaussian.py:372-427)
is the beams' field in their own plane: the same records and sum, with the
per-beam polynomial taken from Q1^-1 and the central ray directly (no model).

``batch_size`` is accepted for signature compatibility; the GPU path needs no
(batch, npix) temporary.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .components import Grid
from .ray import GaussianRay
from .run import _check_model, _device, pack_model

FIELD_DIRECT, FIELD_SEPARABLE, FIELD_DIRECT_F64 = 0, 1, 2
_METHODS = {"direct": FIELD_DIRECT, "separable": FIELD_SEPARABLE, "fp64": FIELD_DIRECT_F64}
EW_NONSEPARABLE = 0x10


class TgBeams(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", C.c_void_p), ("y", C.c_void_p), ("dx", C.c_void_p),
                ("dy", C.c_void_p), ("z", C.c_double), ("pathlength", C.c_void_p),
                ("amplitude", C.c_void_p), ("waist_xy", C.c_void_p), ("radii", C.c_void_p),
                ("wavelength", C.c_void_p), ("wavelength_scalar", C.c_double),
                ("theta", C.c_void_p)]


class TgPixelMap(C.Structure):
    _fields_ = [("h", C.c_int32), ("w", C.c_int32), ("t", C.c_double * 6)]


N.register("tg_field_workspace", C.c_size_t, [C.c_int64, C.c_int32, C.c_int32, C.c_int32])
N.register("tg_field_prep", C.c_int, [C.POINTER(N.TgModel), C.POINTER(TgBeams), C.POINTER(TgPixelMap),
                                      C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p])
N.register("tg_field_prep_input", C.c_int, [C.POINTER(TgBeams), C.POINTER(TgPixelMap), C.c_void_p,
                                            C.c_size_t, C.c_void_p, C.c_void_p])
N.register("tg_decompose_q_inv", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p])
N.register("tg_field_eval", C.c_int, [C.c_int32, C.c_int64, C.POINTER(TgPixelMap), C.c_void_p,
                                      C.c_void_p, C.c_size_t, C.c_void_p])


class TgFieldGrads(C.Structure):
    _fields_ = [("amplitude", C.c_void_p), ("pathlength", C.c_void_p), ("x", C.c_void_p),
                ("y", C.c_void_p), ("dx", C.c_void_p), ("dy", C.c_void_p), ("raw", C.c_void_p)]


N.register("tg_field_vjp_workspace", C.c_size_t, [C.c_int64, C.c_int32, C.c_int32])
N.register("tg_field_vjp", C.c_int, [C.POINTER(N.TgModel), C.POINTER(TgBeams), C.POINTER(TgPixelMap),
                                     C.c_void_p, C.POINTER(TgFieldGrads), C.c_void_p, C.c_size_t, C.c_void_p])
N.register("tg_field_vjp_input", C.c_int, [C.POINTER(TgBeams), C.POINTER(TgPixelMap), C.c_void_p,
                                           C.POINTER(TgFieldGrads), C.c_void_p, C.c_size_t, C.c_void_p])
N.register("tg_field_vjp_workspace_ex", C.c_size_t, [C.c_int32, C.c_int64, C.c_int32, C.c_int32])
N.register("tg_field_vjp_ex", C.c_int, [C.c_int32, C.POINTER(N.TgModel), C.POINTER(TgBeams),
                                        C.POINTER(TgPixelMap), C.c_void_p, C.POINTER(TgFieldGrads),
                                        C.c_void_p, C.c_size_t, C.c_void_p])
N.register("tg_field_vjp_input_ex", C.c_int, [C.c_int32, C.POINTER(TgBeams), C.POINTER(TgPixelMap), C.c_void_p,
                                              C.POINTER(TgFieldGrads), C.c_void_p, C.c_size_t, C.c_void_p])


def _f64(v, n, dev, width=None):
    if isinstance(v, torch.Tensor):
        t = v.detach().to(device=dev, dtype=torch.float64)
    else:
        t = torch.as_tensor(np.asarray(v, dtype=np.float64), device=dev)
    if width is None:
        t = t.reshape(-1)
        if t.numel() == 1 and n != 1:
            t = t.expand(n)
    else:
        t = t.reshape(-1, width)
        if t.shape[0] == 1 and n != 1:
            t = t.expand(n, width)
    return t.contiguous()


def _upload(a: np.ndarray, dev) -> torch.Tensor:
    """Host array -> device tensor: staged in pinned memory and copied on the
    current stream without a host wait when the target is a CUDA device."""
    t = torch.from_numpy(np.ascontiguousarray(a))
    dev = torch.device(dev)
    if dev.type != "cuda":
        return t.to(dev)
    return t.pin_memory().to(dev, non_blocking=True)


def pixel_map(grid: Grid) -> TgPixelMap:
    t = grid.pixels_to_metres_mat
    pm = TgPixelMap()
    pm.h, pm.w = int(grid.shape[0]), int(grid.shape[1])
    for i, v in enumerate((t[0, 0], t[0, 1], t[0, 2], t[1, 0], t[1, 1], t[1, 2])):
        pm.t[i] = float(v)
    return pm


class BeamSet:
    """Device float64 beam parameters of a GaussianRay."""

    def __init__(self, rays: GaussianRay, dev):
        r = rays
        n = r.size
        self.n = n
        zs = np.unique(np.asarray(r.z.detach().cpu() if isinstance(r.z, torch.Tensor) else r.z,
                                  dtype=np.float64).reshape(-1))
        if zs.size > 1:
            raise NotImplementedError("beams must start from one plane (uniform z)")
        self.z = float(zs[0]) if zs.size else 0.0
        a = r.amplitude
        if isinstance(a, torch.Tensor):
            at = a.detach().to(device=dev, dtype=torch.complex64).reshape(-1)
        else:
            at = _upload(np.asarray(a, dtype=np.complex64).reshape(-1), dev)
        if at.numel() == 1 and n != 1:
            at = at.expand(n)
        self.amp = torch.view_as_real(at.contiguous()).contiguous()
        cols = (r.x, r.y, r.dx, r.dy, r.pathlength, r.wavelength, r.theta)
        pairs = (r.waist_xy, r.radii_of_curv)
        if any(isinstance(v, torch.Tensor) for v in cols + pairs):
            self.x, self.y, self.dx, self.dy, self.pl, self.wl, self.theta = (_f64(v, n, dev) for v in cols)
            self.waist, self.radii = (_f64(v, n, dev, 2) for v in pairs)
            return
        # host values: packed into one float64 buffer (pinned, from the caching
        # host allocator: no fresh pages to fault in), one copy to the device,
        # and every field a contiguous view of it
        dev = torch.device(dev)
        staging = torch.empty(11 * n, dtype=torch.float64, pin_memory=dev.type == "cuda")
        host = staging.numpy()
        for i, v in enumerate(cols):
            a1 = np.asarray(v, dtype=np.float64).reshape(-1)
            host[i * n:(i + 1) * n] = a1 if a1.size != 1 else np.broadcast_to(a1, (n,))
        for i, v in enumerate(pairs):
            a2 = np.asarray(v, dtype=np.float64).reshape(-1, 2)
            host[(7 + 2 * i) * n:(9 + 2 * i) * n] = (a2 if a2.shape[0] != 1 else
                                                     np.broadcast_to(a2, (n, 2))).reshape(-1)
        buf = staging.to(dev, non_blocking=True) if dev.type == "cuda" else staging
        self.x, self.y, self.dx, self.dy, self.pl, self.wl, self.theta = (buf[i * n:(i + 1) * n]
                                                                        for i in range(7))
        self.waist = buf[7 * n:9 * n].view(n, 2)
        self.radii = buf[9 * n:11 * n].view(n, 2)

    def struct(self) -> TgBeams:
        b = TgBeams()
        b.n = self.n
        b.x, b.y, b.dx, b.dy = (t.data_ptr() for t in (self.x, self.y, self.dx, self.dy))
        b.z = self.z
        b.pathlength = self.pl.data_ptr()
        b.amplitude = self.amp.data_ptr()
        b.waist_xy = self.waist.data_ptr()
        b.radii = self.radii.data_ptr()
        b.wavelength = self.wl.data_ptr()
        b.wavelength_scalar = 0.0
        b.theta = self.theta.data_ptr()
        return b


class FieldPlan:
    """Prepared beams + workspace for repeated field evaluations.

    ``model``: component list ending in the detector Grid (the detector field,
    gaussian.py:225-273); or ``model=None`` with ``grid=`` for the field of
    the beams in their own plane (gaussian.py:372-427)."""

    def __init__(self, gaussian_rays: GaussianRay, model, method: str = "auto", *, grid=None):
        if not isinstance(gaussian_rays, GaussianRay):
            raise TypeError("gaussian_rays must be a GaussianRay (gaussian.py:228)")
        comps = None
        if model is None:
            if not isinstance(grid, Grid):
                raise ValueError("the input-plane field needs a Grid (gaussian.py:377-381)")
        else:
            comps = _check_model(model)
            grid = comps[-1]
            if not isinstance(grid, Grid):
                raise ValueError("the last model element must be a Detector grid (gaussian.py:231-232)")
        self.dev = _device()
        self.beams = BeamSet(gaussian_rays, self.dev)
        self.pm = pixel_map(grid)
        self.shape = (int(grid.shape[0]), int(grid.shape[1]))
        sizes = [N.lib().tg_field_workspace(self.beams.n, self.pm.h, self.pm.w, m) for m in (0, 1, 2)]
        self.ws = torch.empty(max(sizes) + 256, dtype=torch.uint8, device=self.dev)
        off = (-self.ws.data_ptr()) % 256
        self.ws_ptr = self.ws.data_ptr() + off
        self.ws_bytes = self.ws.numel() - off
        self.flags = torch.zeros(1, dtype=torch.int32, device=self.dev)
        if comps is None:
            st = N.lib().tg_field_prep_input(C.byref(self.beams.struct()), C.byref(self.pm), self.ws_ptr,
                                             self.ws_bytes, self.flags.data_ptr(), N.stream_ptr())
            N.check(st, "tg_field_prep_input")
        else:
            m, keep = pack_model(comps)
            st = N.lib().tg_field_prep(C.byref(m), C.byref(self.beams.struct()), C.byref(self.pm),
                                       self.ws_ptr, self.ws_bytes, self.flags.data_ptr(), N.stream_ptr())
            del keep
            N.check(st, "tg_field_prep")
        if method == "auto":
            method = "separable" if int(self.flags.item()) == 0 else "direct"
        if method not in _METHODS:
            raise ValueError(f"unknown method {method!r}")
        self.method = method
        self.out = torch.empty(self.shape, dtype=torch.complex64, device=self.dev)
        self.comps = comps
        self._vjp_ws = None

    def evaluate(self, method: str | None = None, out: torch.Tensor | None = None) -> torch.Tensor:
        method = method or self.method
        o = self.out if out is None else out
        st = N.lib().tg_field_eval(_METHODS[method], self.beams.n, C.byref(self.pm),
                                   torch.view_as_real(o).data_ptr(), self.ws_ptr, self.ws_bytes,
                                   N.stream_ptr())
        N.check(st, "tg_field_eval")
        return o

    @property
    def separable(self) -> bool:
        return int(self.flags.item()) == 0

    def vjp(self, grad: torch.Tensor, beams: bool = True, model: bool = True, method: str | None = None) -> dict:
        """Gradients of a real loss L from its gradient with respect to the
        field, ``grad`` = dL/dRe F + i dL/dIm F (complex (H, W), PyTorch's
        convention): per beam ``amplitude`` (complex64), ``pathlength``,
        ``x``, ``y``, ``dx``, ``dy`` (float64) when ``beams``, and the model's
        per-step sums ``raw`` (float64 [2 * components, 4], the layout of the
        trace adjoint) when ``model`` (tg_field_vjp_ex / tg_field_vjp_input_ex).
        ``method`` ("separable" or "direct", default: the plan's) picks how the
        per-beam moments are formed: a GEMM on the tensor cores for separable
        beams, or the direct pass over beams x pixels."""
        n, dev = self.beams.n, self.dev
        method = method or self.method
        code = FIELD_SEPARABLE if method == "separable" else FIELD_DIRECT
        g = torch.view_as_real(grad.to(device=dev, dtype=torch.complex64).reshape(self.shape).contiguous())
        nb = N.lib().tg_field_vjp_workspace_ex(code, n, self.pm.h, self.pm.w)
        if self._vjp_ws is None or self._vjp_ws.numel() < nb + 256:
            self._vjp_ws = torch.empty(nb + 256, dtype=torch.uint8, device=dev)
        ws = self._vjp_ws
        off = (-ws.data_ptr()) % 256
        res = {}
        out = TgFieldGrads()
        if beams:
            res["amplitude"] = torch.empty(n, dtype=torch.complex64, device=dev)
            out.amplitude = torch.view_as_real(res["amplitude"]).data_ptr()
            for k in ("pathlength", "x", "y", "dx", "dy"):
                res[k] = torch.empty(n, dtype=torch.float64, device=dev)
                setattr(out, k, res[k].data_ptr())
        if model and self.comps is not None:
            res["raw"] = torch.empty((2 * len(self.comps), 4), dtype=torch.float64, device=dev)
            out.raw = res["raw"].data_ptr()
        if self.comps is None:
            st = N.lib().tg_field_vjp_input_ex(code, C.byref(self.beams.struct()), C.byref(self.pm),
                                               g.data_ptr(), C.byref(out), ws.data_ptr() + off,
                                               ws.numel() - off, N.stream_ptr())
            N.check(st, "tg_field_vjp_input_ex")
        else:
            m, keep = pack_model(self.comps)
            st = N.lib().tg_field_vjp_ex(code, C.byref(m), C.byref(self.beams.struct()), C.byref(self.pm),
                                         g.data_ptr(), C.byref(out), ws.data_ptr() + off, ws.numel() - off,
                                         N.stream_ptr())
            del keep
            N.check(st, "tg_field_vjp_ex")
        return res


_BEAM_FIELDS = ("amplitude", "pathlength", "x", "y", "dx", "dy")


class _FieldFn(torch.autograd.Function):
    """The detector (or input-plane) field with its hand-written adjoint:
    forward through FieldPlan.evaluate, backward through FieldPlan.vjp."""

    @staticmethod
    def forward(ctx, spec, *inputs):
        plan = spec["plan"]
        ctx.spec = spec
        return plan.evaluate(spec["method"]).clone()

    @staticmethod
    def backward(ctx, grad):
        spec = ctx.spec
        plan = spec["plan"]
        r = plan.vjp(grad, beams=bool(spec["beam_inputs"]), model=bool(spec["params"]))
        out = []
        for name, t in spec["beam_inputs"]:
            if t is None:
                out.append(None)
                continue
            g = r[name]
            if t.numel() == 1 and g.numel() != 1:
                g = g.sum()
            out.append(g.to(t.dtype).reshape(t.shape))
        if spec["params"]:
            from .run import param_gradient
            for (i, path, t) in spec["params"]:
                out.append(param_gradient(plan.comps, i, path, r["raw"]).to(t.dtype).reshape(t.shape))
        return (None, *out)


def _field_autograd(gaussian_rays: GaussianRay, model, method: str, grid=None):
    """The field through _FieldFn when a beam field (amplitude, pathlength,
    x, y, dx, dy) or a model parameter tensor requires grad, else None."""
    if not torch.is_grad_enabled():
        return None
    from .run import _grad_params
    beam_inputs = []
    for name in _BEAM_FIELDS:
        v = getattr(gaussian_rays, name)
        beam_inputs.append((name, v if isinstance(v, torch.Tensor) and v.requires_grad else None))
    params = _grad_params(_check_model(model)) if model is not None else []
    if not params and all(t is None for _, t in beam_inputs):
        return None
    plan = FieldPlan(gaussian_rays, model, method, grid=grid)
    spec = {"plan": plan, "method": plan.method, "beam_inputs": beam_inputs, "params": params}
    tensors = [t for _, t in beam_inputs if t is not None] + [t for (_, _, t) in params]
    spec["beam_inputs"] = [(n_, t) for n_, t in beam_inputs if t is not None]
    return _FieldFn.apply(spec, *tensors)


def make_gaussian_image(gaussian_rays: GaussianRay, model, batch_size: int = 128,
                        method: str = "auto") -> torch.Tensor:
    """Complex64 detector field (H, W) of the Gaussian beamlets after ``model``
    (gaussian.py:225-273).  Differentiable (hand-written adjoint,
    tg_field_vjp) with respect to the beams' amplitude, pathlength, x, y, dx,
    dy and the model's parameter tensors that require grad."""
    out = _field_autograd(gaussian_rays, model, method)
    if out is not None:
        return out
    plan = FieldPlan(gaussian_rays, model, method)
    return plan.evaluate().clone()


def evaluate_gaussian_input_image(gaussian_rays: GaussianRay, grid, batch_size: int = 128,
                                  method: str = "auto") -> torch.Tensor:
    """Complex64 field (H, W) of the Gaussian beamlets in their own plane,
    sampled at the pixel centres of ``grid`` (gaussian.py:372-400).
    Differentiable with respect to the beams' amplitude, pathlength, x, y,
    dx, dy (tg_field_vjp_input)."""
    out = _field_autograd(gaussian_rays, None, method, grid=grid)
    if out is not None:
        return out
    plan = FieldPlan(gaussian_rays, None, method, grid=grid)
    return plan.evaluate().clone()


def decompose_Q_inv(Q_inv, wavelength, eps: float = 1e-12):
    """gaussian.py:35-89: (waist_x, waist_y, r_x, r_y, theta) of 2x2 complex
    Q^-1 matrices (leading batch axes allowed), the major axis first.  theta
    equals the reference's up to a multiple of pi."""
    dev = _device()
    q = Q_inv if isinstance(Q_inv, torch.Tensor) else torch.as_tensor(np.asarray(Q_inv, np.complex128))
    q = q.to(device=dev, dtype=torch.complex128)
    batch = tuple(q.shape[:-2])
    q = q.reshape(-1, 2, 2).contiguous()
    n = q.shape[0]
    wl = torch.as_tensor(wavelength, dtype=torch.float64)
    wl_t = None
    if wl.numel() > 1:
        if wl.numel() != n:
            raise ValueError("wavelength must be a scalar or one value per matrix")
        wl_t = wl.to(dev).reshape(-1).contiguous()
    waist = torch.empty((n, 2), dtype=torch.float64, device=dev)
    radii = torch.empty((n, 2), dtype=torch.float64, device=dev)
    theta = torch.empty(n, dtype=torch.float64, device=dev)
    N.check(N.lib().tg_decompose_q_inv(n, torch.view_as_real(q).data_ptr(), N.ptr(wl_t),
                                       float(wl.reshape(-1)[0]) if wl_t is None else 0.0, float(eps),
                                       waist.data_ptr(), radii.data_ptr(), theta.data_ptr(),
                                       N.stream_ptr()), "tg_decompose_q_inv")
    rs = lambda t: t.reshape(batch) if batch else t.reshape(())  # noqa: E731
    return rs(waist[:, 0]), rs(waist[:, 1]), rs(radii[:, 0]), rs(radii[:, 1]), rs(theta)


N.register("tg_beam_q_inv", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                      C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p])
N.register("tg_qinv_abcd", C.c_int, [C.c_int64] + [C.c_void_p] * 7)
N.register("tg_beam_profile", C.c_int, [C.c_int64] + [C.c_void_p] * 9)
N.register("tg_gaussian_beam", C.c_int, [C.c_int64] + [C.c_void_p] * 8)


def beam_q_inv(rays: GaussianRay, full: bool):
    """GaussianRay.q_inv (``full=False``: the per-axis 1/qx, 1/qy, each (n,))
    and GaussianRay.Q_inv (``full=True``: (n, 2, 2) = R diag R^T), complex128
    on the device (gaussian.py:138-177)."""
    dev = _device()
    n = rays.size
    waist = _f64(rays.waist_xy, n, dev, 2)
    radii = _f64(rays.radii_of_curv, n, dev, 2)
    wl = _f64(rays.wavelength, n, dev)
    theta = _f64(rays.theta, n, dev)
    if full:
        out = torch.empty((n, 2, 2), dtype=torch.complex128, device=dev)
        qxy_p, q_p = None, torch.view_as_real(out).data_ptr()
    else:
        out = torch.empty((n, 2), dtype=torch.complex128, device=dev)
        qxy_p, q_p = torch.view_as_real(out).data_ptr(), None
    N.check(N.lib().tg_beam_q_inv(n, waist.data_ptr(), radii.data_ptr(), wl.data_ptr(), 0.0,
                                  theta.data_ptr(), 0.0, qxy_p, q_p, N.stream_ptr()), "tg_beam_q_inv")
    if full:
        return out
    if np.ndim(rays.waist_xy) <= 1:  # one beam given as (2,): scalars, as waist_xy.T unpacks
        return out[0, 0], out[0, 1]
    return out[:, 0], out[:, 1]


def _dev_tensor(v, dtype, dev):
    if isinstance(v, torch.Tensor):
        return v.detach().to(device=dev, dtype=dtype)
    npt = np.complex128 if dtype == torch.complex128 else np.float64
    return torch.as_tensor(np.asarray(v, dtype=npt), device=dev)


def Qinv_ABCD(Qinv, A, B, C, D):  # noqa: N803 - the reference's names (ctypes unused here)
    """gaussian.py:92-96: (A + B Q)^-1 (C + D Q) for 2x2 blocks with leading
    batch axes (broadcast), Q complex, A-D real; complex128 on the device."""
    dev = _device()
    q = _dev_tensor(Qinv, torch.complex128, dev)
    mats = []
    for m in (A, B, C, D):
        t = m.detach() if isinstance(m, torch.Tensor) else torch.as_tensor(np.asarray(m))
        if t.is_complex():
            if bool((t.imag != 0).any()):
                raise NotImplementedError("Qinv_ABCD takes real A, B, C, D (ABCD matrices are real)")
            t = t.real
        mats.append(t.to(device=dev, dtype=torch.float64))
    if any(t.shape[-2:] != (2, 2) for t in [q] + mats):
        raise ValueError("Qinv_ABCD needs 2x2 blocks in the last two axes")
    batch = torch.broadcast_shapes(*(t.shape[:-2] for t in [q] + mats))
    q = q.expand(*batch, 2, 2).reshape(-1, 2, 2).contiguous()
    mats = [t.expand(*batch, 2, 2).reshape(-1, 2, 2).contiguous() for t in mats]
    n = q.shape[0]
    out = torch.empty((n, 2, 2), dtype=torch.complex128, device=dev)
    N.check(N.lib().tg_qinv_abcd(n, torch.view_as_real(q).data_ptr(), *(t.data_ptr() for t in mats),
                                 torch.view_as_real(out).data_ptr(), N.stream_ptr()), "tg_qinv_abcd")
    return out.reshape(*batch, 2, 2)


def _profile(which: str, z=None, w0=None, wl=None, z_r=None):
    dev = _device()
    given = {k: _dev_tensor(v, torch.float64, dev) for k, v in
             (("z", z), ("w0", w0), ("wl", wl), ("z_r", z_r)) if v is not None}
    shape = torch.broadcast_shapes(*(t.shape for t in given.values()))
    flat = {k: t.expand(shape).reshape(-1).contiguous() for k, t in given.items()}
    n = int(np.prod(shape)) if len(shape) else 1
    out = torch.empty(n, dtype=torch.complex128 if which == "q_inv" else torch.float64, device=dev)
    optr = torch.view_as_real(out).data_ptr() if which == "q_inv" else out.data_ptr()
    outs = {k: (optr if k == which else None) for k in ("z_r_out", "w_z", "r", "q_inv")}
    p = lambda k: flat[k].data_ptr() if k in flat else None  # noqa: E731
    N.check(N.lib().tg_beam_profile(n, p("z"), p("w0"), p("wl"), p("z_r"), outs["z_r_out"], outs["w_z"],
                                    outs["r"], outs["q_inv"], N.stream_ptr()), "tg_beam_profile")
    return out.reshape(shape)


def zR(w0, wavelength):
    """Rayleigh range pi w0^2 / wavelength (gaussian.py:17-18), on the device."""
    return _profile("z_r_out", w0=w0, wl=wavelength)


def w_z(w0, z, z_r):
    """Beam radius w0 sqrt(1 + (z / z_r)^2) (gaussian.py:13-14), on the device."""
    return _profile("w_z", z=z, w0=w0, z_r=z_r)


def R(z, z_r):
    """Wavefront radius z (1 + (z_r / z)^2), infinite for |z| < 1e-10
    (gaussian.py:21-28), on the device."""
    return _profile("r", z=z, z_r=z_r)


def q_inv(z, w0, wl):
    """Complex 1/q of a beam of waist w0 at distance z from its focus
    (gaussian.py:99-109), elementwise, on the device."""
    return _profile("q_inv", z=z, w0=w0, wl=wl)


def gaussian_beam(x, y, q_inv, k, offset_x=0, offset_y=0):
    """exp(1j k ((x + offset_x)^2 + (y + offset_y)^2) / 2 q_inv)
    (gaussian.py:31-32), elementwise, complex128 on the device."""
    dev = _device()
    ts = [_dev_tensor(v, torch.float64, dev) for v in (x, y, k, offset_x, offset_y)]
    q = _dev_tensor(q_inv, torch.complex128, dev)
    shape = torch.broadcast_shapes(q.shape, *(t.shape for t in ts))
    xs, ys, ks, oxs, oys = (t.expand(shape).reshape(-1).contiguous() for t in ts)
    qs = q.expand(shape).reshape(-1).contiguous()
    n = xs.numel()
    out = torch.empty(n, dtype=torch.complex128, device=dev)
    N.check(N.lib().tg_gaussian_beam(n, xs.data_ptr(), ys.data_ptr(), torch.view_as_real(qs).data_ptr(),
                                     ks.data_ptr(), oxs.data_ptr(), oys.data_ptr(),
                                     torch.view_as_real(out).data_ptr(), N.stream_ptr()), "tg_gaussian_beam")
    return out.reshape(shape)


def fibonacci_spiral(nb_samples: int, radius: float, alpha=2):
    """Golden-angle (Vogel) spiral sample positions in a disc (utils.py:297-325)."""
    ga = np.pi * (3.0 - np.sqrt(5.0))
    nbd = np.round(alpha * np.sqrt(nb_samples))
    ii = np.arange(nb_samples)
    rr = np.where(ii > nb_samples - (nbd + 1), radius,
                  radius * np.sqrt((ii + 0.5) / (nb_samples - 0.5 * (nbd + 1))))
    rr[0] = 0.0
    phi = ii * ga
    return rr * np.cos(phi), rr * np.sin(phi)


N.register("tg_misaligned_gaussian_workspace", C.c_size_t, [C.c_int64, C.c_int64])
N.register("tg_propagate_misaligned_gaussian", C.c_int,
           [C.c_int64] + [C.c_void_p] * 12 + [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                              C.c_void_p])
N.register("tg_evaluate_misaligned_input_gaussian", C.c_int,
           [C.c_int64] + [C.c_void_p] * 6 + [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                             C.c_void_p])


def _per_beam(v, n, tail, dtype, dev):
    """(n, *tail) contiguous device tensor; a value without the beam axis is
    broadcast to every beam."""
    t = _dev_tensor(v, dtype, dev)
    return t.expand(n, *tail).contiguous() if t.dim() < 1 + len(tail) else t.reshape(n, *tail).contiguous()


def _points(r, dev):
    t = _dev_tensor(r, torch.float64, dev).reshape(-1, 2).contiguous()
    return t, t.shape[0]


def _run_points(fn, n, npts, dev, args, r):
    out = torch.empty(npts, dtype=torch.complex128, device=dev)
    if n == 0 or npts == 0:
        out.zero_()
        return out
    ws = torch.empty(N.lib().tg_misaligned_gaussian_workspace(n, npts), dtype=torch.uint8, device=dev)
    ptrs = [torch.view_as_real(a).data_ptr() if a.is_complex() else a.data_ptr() for a in args]
    N.check(getattr(N.lib(), fn)(n, *ptrs, npts, r.data_ptr(), torch.view_as_real(out).data_ptr(),
                                 ws.data_ptr(), ws.numel(), N.stream_ptr()), fn)
    return out


def propagate_misaligned_gaussian_jax_scan(amp, phase_offset, Q1_inv, A, B, C, D, e, f, r1m, theta1m,  # noqa: N803
                                           k, r2, batch_size=128):
    """gaussian.py:319-337: the field of n beams with per-beam ABCD blocks
    (A, B, C, D: (n, 2, 2); e, f, r1m, theta1m: (n, 2); amp, phase_offset, k:
    (n,)) at the points r2 (npix, 2) = (x, y), summed over beams; complex128
    (npix,) on the device, every term in float64.  ``batch_size`` is accepted
    for signature compatibility (the kernel needs no (batch, npix) temporary)."""
    dev = _device()
    a = _dev_tensor(amp, torch.complex128, dev).reshape(-1).contiguous()
    n = a.numel()
    args = [a, _per_beam(phase_offset, n, (), torch.float64, dev),
            _per_beam(Q1_inv, n, (2, 2), torch.complex128, dev)]
    args += [_per_beam(m, n, (2, 2), torch.float64, dev) for m in (A, B, C, D)]
    args += [_per_beam(v, n, (2,), torch.float64, dev) for v in (e, f, r1m, theta1m)]
    args.append(_per_beam(k, n, (), torch.float64, dev))
    r, npts = _points(r2, dev)
    return _run_points("tg_propagate_misaligned_gaussian", n, npts, dev, args, r)


def evaluate_misaligned_input_gaussian_jax_scan(amp, phase_offset, Q1_inv, r1m, theta1m, k, r1,  # noqa: N803
                                                batch_size=128):
    """gaussian.py:410-427: the field of n beams in their own plane at the
    points r1 (npix, 2) = (x, y); complex128 (npix,) on the device."""
    dev = _device()
    a = _dev_tensor(amp, torch.complex128, dev).reshape(-1).contiguous()
    n = a.numel()
    args = [a, _per_beam(phase_offset, n, (), torch.float64, dev),
            _per_beam(Q1_inv, n, (2, 2), torch.complex128, dev),
            _per_beam(r1m, n, (2,), torch.float64, dev), _per_beam(theta1m, n, (2,), torch.float64, dev),
            _per_beam(k, n, (), torch.float64, dev)]
    r, npts = _points(r1, dev)
    return _run_points("tg_evaluate_misaligned_input_gaussian", n, npts, dev, args, r)


def _einsum(spec, *ops):
    if any(isinstance(o, torch.Tensor) for o in ops):
        return torch.einsum(spec, *(torch.as_tensor(o) for o in ops))
    return np.einsum(spec, *ops)


def matrix_vector_mul(M, v):
    """gaussian.py:180-187: M @ v for one 2x2 block and one 2-vector."""
    return _einsum("ij,j->i", M, v)


def matrix_matrix_mul(M1, M2):
    """gaussian.py:190-197: M1 @ M2 for 2x2 blocks."""
    return _einsum("ij,jk->ik", M1, M2)


def matrix_quadratic_mul(v, M):
    """gaussian.py:200-207: v^T M v."""
    return _einsum("i,ij,j->", v, M, v)


def matrix_linear_mul(v, M, w):
    """gaussian.py:210-218: v^T M w_n for every row w_n of w (np, 2)."""
    return _einsum("i,ij,nj->n", v, M, w)


def matrix_matrix_matrix_mul(M1, M2, M3):
    """gaussian.py:221-222: M1 M2 M3^T per batch entry (n, 2, 2)."""
    return _einsum("nij,njk,npk->nip", M1, M2, M3)
