"""Model execution (drop-in for temgym_core.run, run.py:17-267).

``run_to_end`` packs the model into the C-ABI component table and makes ONE
fused kernel launch over all rays (forward), or, under autograd, registers
the recompute-based adjoint kernel as the backward.  There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Sequence

import numpy as np
import torch

from . import _native as N
from .components import Component, Descanner, Grid, ThickLens, Source, _f
from .propagator import FreeSpaceParaxial, Propagator
from .ray import Ray, as_f32, as_f64_or_scalar


# ----------------------------------------------------------------- packing

def _check_model(model) -> list:
    comps = list(model)
    for c in comps:
        if not isinstance(c, (Component, Source)):
            raise NotImplementedError(
                f"{type(c).__name__} is not a built-in component; the GPU path has no "
                "generic-callable fallback")
    if len(comps) > N.MAX_COMPONENTS:
        raise ValueError(f"model has {len(comps)} components; the maximum is {N.MAX_COMPONENTS}")
    return comps


def _prop_code(propagator) -> int:
    """C-ABI propagator selector (TG_PROP_*) of a propagator object."""
    from .propagator import FreeSpaceDirCosine
    if propagator is None or isinstance(propagator, FreeSpaceParaxial):
        return N.PROP_PARAXIAL
    if isinstance(propagator, FreeSpaceDirCosine):
        return N.PROP_DIRCOS
    raise NotImplementedError(f"{type(propagator).__name__} is not a GPU propagator")


def pack_model(model, propagator=None):
    """(TgModel, keep-alive array) for a sequence of components; ``propagator``
    selects the free-space model between them (default paraxial)."""
    comps = _check_model(model)
    arr = (N.TgComponent * max(1, len(comps)))()
    for i, c in enumerate(comps):
        c._pack(arr[i])
    m = N.TgModel()
    m.n_components = len(comps)
    m.propagator = _prop_code(propagator)
    m.components = C.cast(arr, C.POINTER(N.TgComponent))
    return m, arr


def _rays_struct(n, x, y, dx, dy, z_t, z_s, pl_t, pl_s, amp=None) -> N.TgRays:
    r = N.TgRays()
    r.n = n
    r.x, r.y, r.dx, r.dy = N.ptr(x), N.ptr(y), N.ptr(dx), N.ptr(dy)
    r.z = N.ptr(z_t)
    r.z_scalar = z_s
    r.pathlength = N.ptr(pl_t)
    r.pl_scalar = pl_s
    r.amplitude = N.ptr(amp)
    return r


class _Soa:
    """Device structure-of-arrays view of a Ray."""

    def __init__(self, ray: Ray, device):
        n = ray.size
        self.n = n
        self.x = as_f32(ray.x, n, device)
        self.y = as_f32(ray.y, n, device)
        self.dx = as_f32(ray.dx, n, device)
        self.dy = as_f32(ray.dy, n, device)
        self.z_t, self.z_s = as_f64_or_scalar(ray.z, n, device)
        self.pl_t, self.pl_s = as_f64_or_scalar(ray.pathlength, n, device)
        amp = getattr(ray, "amplitude", None)
        self.amp = None
        if amp is not None and not isinstance(amp, complex) and not np.iscomplexobj(np.asarray(
                amp.detach().cpu() if isinstance(amp, torch.Tensor) else amp)):
            self.amp = as_f32(amp, n, device)

    def struct(self) -> N.TgRays:
        return _rays_struct(self.n, self.x, self.y, self.dx, self.dy, self.z_t, self.z_s,
                            self.pl_t, self.pl_s, self.amp)


def _ray_scalar_input(ray: Ray) -> bool:
    return all(not isinstance(getattr(ray, f), (torch.Tensor, np.ndarray)) or
               getattr(ray, f).ndim == 0 for f in ("x", "y", "dx", "dy"))


def _fwd_launch(model, soa: _Soa, grid=None, want_pix=False, hist=None, want_amp=False, propagator=None):
    dev = soa.x.device
    n = soa.n
    o4 = torch.empty((4, n), dtype=torch.float32, device=dev)  # one allocation, four views
    ox, oy, odx, ody = o4[0], o4[1], o4[2], o4[3]
    opl = torch.empty(n, dtype=torch.float64, device=dev)
    oamp = torch.empty(n, dtype=torch.float32, device=dev) if (want_amp or soa.amp is not None) else None
    m, keep = pack_model(model, propagator)
    out = _rays_struct(n, ox, oy, odx, ody, None, 0.0, opl, 0.0, oamp)
    zout = C.c_double(0.0)
    py = px = None
    g = None
    if grid is not None:
        g = grid._tg_grid()
        if want_pix:
            pyx = torch.empty((2, n), dtype=torch.int32, device=dev)  # one allocation, two views
            py, px = pyx[0], pyx[1]
    if hist is not None and hist.dtype not in (torch.int32, torch.int64):
        raise TypeError("histogram accumulator must be int32 or int64")
    lib = N.lib()
    # many rays per pixel: per-SM shared-memory histograms summed at the end
    ws_bytes = lib.tg_trace_image_workspace(n, C.byref(g)) if (hist is not None and g is not None) else 0
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev) if ws_bytes else None
    st = lib.tg_trace_image(C.byref(m), C.byref(soa.struct()), C.byref(out), C.byref(zout),
                            C.byref(g) if g is not None else None, N.ptr(py), N.ptr(px),
                            N.ptr(hist), 1 if (hist is not None and hist.dtype == torch.int64) else 0,
                            N.ptr(ws), ws_bytes, N.stream_ptr())
    del keep
    N.check(st, "tg_trace_image")
    return ox, oy, odx, ody, opl, zout.value, oamp, py, px


# ---------------------------------------------------------- differentiable

_DESCAN_FIELDS = ("pxo_pxi", "pxo_pyi", "pyo_pxi", "pyo_pyi", "sxo_pxi", "sxo_pyi", "syo_pxi",
                  "syo_pyi", "offpxi", "offpyi", "offsxi", "offsyi", "pxo_sxi", "pxo_syi",
                  "pyo_sxi", "pyo_syi", "sxo_sxi", "sxo_syi", "syo_sxi", "syo_syi")
# DescanError field -> (row, col) of the 4x4 matrix, or ("off", row)
_DESCAN_POS = {"pxo_pxi": (0, 0), "pxo_pyi": (0, 1), "pyo_pxi": (1, 0), "pyo_pyi": (1, 1),
               "sxo_pxi": (2, 0), "sxo_pyi": (2, 1), "syo_pxi": (3, 0), "syo_pyi": (3, 1),
               "offpxi": ("off", 0), "offpyi": ("off", 1), "offsxi": ("off", 2),
               "offsyi": ("off", 3), "pxo_sxi": (0, 2), "pxo_syi": (0, 3), "pyo_sxi": (1, 2),
               "pyo_syi": (1, 3), "sxo_sxi": (2, 2), "sxo_syi": (2, 3), "syo_sxi": (3, 2),
               "syo_syi": (3, 3)}


def _grad_params(comps) -> list:
    """(component index, path, tensor) for every parameter tensor needing grad."""
    out = []
    for i, c in enumerate(comps):
        names = [f for f in getattr(c, "__dataclass_fields__", {})]
        for name in names:
            v = getattr(c, name)
            if isinstance(v, torch.Tensor) and v.requires_grad:
                out.append((i, name, v))
            if name == "descan_error":
                for dn in _DESCAN_FIELDS:
                    dv = getattr(v, dn)
                    if isinstance(dv, torch.Tensor) and dv.requires_grad:
                        out.append((i, "descan_error." + dn, dv))
    return out


def param_gradient(comps, i, path, raw):
    """dL/d(parameter) from the adjoint's per-step sums raw[(2*n_components), 4]."""
    c = comps[i]
    nc = len(comps)
    comp = raw[2 * i + 1]
    if path in ("z", "z_po"):
        g = raw[2 * i, 0]
        if i + 1 < nc and not isinstance(c, ThickLens):
            g = g - raw[2 * i + 2, 0]
        return g
    if path == "z_pi":
        return -raw[2 * i + 2, 0] if i + 1 < nc else raw[0, 0] * 0.0
    if path == "focal_length" or path == "def_x":
        return comp[0]
    if path == "def_y":
        return comp[1]
    if path == "angle":
        return comp[0] * (math.pi / 180.0)
    if isinstance(c, Descanner):
        m = torch.as_tensor(c.descan_error.as_matrix4(), dtype=torch.float64, device=raw.device)
        s = [_f(c.scan_pos_x), _f(c.scan_pos_y), _f(c.scan_tilt_x), _f(c.scan_tilt_y)]
        g4 = comp[0:4]
        sp = {"scan_pos_x": 0, "scan_pos_y": 1, "scan_tilt_x": 2, "scan_tilt_y": 3}
        if path in sp:
            j = sp[path]
            return (g4 * m[:, j]).sum() - g4[j]
        dn = path.split(".", 1)[1]
        pos = _DESCAN_POS[dn]
        if pos[0] == "off":
            return g4[pos[1]]
        return g4[pos[0]] * s[pos[1]]
    sp = {"scan_pos_x": 0, "scan_pos_y": 1, "scan_tilt_x": 2, "scan_tilt_y": 3}
    if path in sp:
        return comp[sp[path]]
    raise NotImplementedError(f"no gradient rule for {type(c).__name__}.{path}")


class _TraceFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, spec, x, y, dx, dy, pl, zin, *params):
        comps, soa = spec["comps"], spec["soa"]
        ox, oy, odx, ody, opl, zout, _, _, _ = _fwd_launch(comps, soa, propagator=spec["propagator"])
        spec["zout"] = zout
        ctx.spec = spec
        return ox, oy, odx, ody, opl

    @staticmethod
    def backward(ctx, gx, gy, gdx, gdy, gpl):
        spec = ctx.spec
        comps, soa, plist = spec["comps"], spec["soa"], spec["params"]
        n = soa.n
        dev = soa.x.device
        z32 = lambda: torch.zeros(n, dtype=torch.float32, device=dev)  # noqa: E731
        gx = z32() if gx is None else gx.to(torch.float32).contiguous()
        gy = z32() if gy is None else gy.to(torch.float32).contiguous()
        gdx = z32() if gdx is None else gdx.to(torch.float32).contiguous()
        gdy = z32() if gdy is None else gdy.to(torch.float32).contiguous()
        gpl = None if gpl is None else gpl.to(torch.float64).contiguous()
        ix, iy, idx, idy = z32(), z32(), z32(), z32()
        ipl = torch.empty(n, dtype=torch.float64, device=dev)
        need_raw = bool(plist) or spec["z_grad"]
        m, keep = pack_model(comps, spec["propagator"])
        raw = torch.zeros((2 * len(comps), 4), dtype=torch.float64, device=dev) if need_raw else None
        ws = None
        if need_raw:
            nbytes = N.lib().tg_trace_vjp_workspace(n, C.byref(m))
            ws = torch.empty(max(8, nbytes), dtype=torch.uint8, device=dev)
        gout = _rays_struct(n, gx, gy, gdx, gdy, None, 0.0, gpl, 0.0)
        gin = _rays_struct(n, ix, iy, idx, idy, None, 0.0, ipl, 0.0)
        st = N.lib().tg_trace_vjp(C.byref(m), C.byref(soa.struct()), C.byref(gout), C.byref(gin),
                                  N.ptr(raw), N.ptr(ws), 0 if ws is None else ws.numel(),
                                  N.stream_ptr())
        del keep
        N.check(st, "tg_trace_vjp")
        pgrads = []
        for (i, path, t) in plist:
            g = param_gradient(comps, i, path, raw)
            pgrads.append(g.to(t.dtype).reshape(t.shape))
        gz = (-raw[0, 0]).reshape(()) if (spec["z_grad"] and raw is not None and len(comps)) else None
        shape = spec["shape"]
        if gpl is None:
            ipl = None
        return (None, ix.reshape(shape), iy.reshape(shape), idx.reshape(shape),
                idy.reshape(shape), ipl if ipl is None else ipl.reshape(shape), gz, *pgrads)


def _needs_grad(ray, comps) -> bool:
    if not torch.is_grad_enabled():
        return False
    for f in ("x", "y", "dx", "dy", "pathlength", "z"):
        v = getattr(ray, f)
        if isinstance(v, torch.Tensor) and v.requires_grad:
            return True
    return bool(_grad_params(comps))


def _in_shape(ray: Ray):
    return () if _ray_scalar_input(ray) else (ray.size,)


def _device():
    N.require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def run_to_end(ray: Ray, components: Sequence[Component],
               propagator=FreeSpaceParaxial()) -> Ray:
    """Propagate rays through every component (run.py:85-116), one fused
    GPU launch.  Returns a Ray with float32 x, y, dx, dy, float64 pathlength
    and uniform z.  ``propagator``: FreeSpaceParaxial (default) or
    FreeSpaceDirCosine (propagator.py:79-116)."""
    _prop_code(propagator)
    comps = _check_model(components)
    dev = _device()
    soa = _Soa(ray, dev)
    shape = _in_shape(ray)
    if _needs_grad(ray, comps):
        plist = _grad_params(comps)
        zt = ray.z if isinstance(ray.z, torch.Tensor) and ray.z.requires_grad and ray.z.dim() == 0 else None
        spec = {"comps": comps, "soa": soa, "params": plist, "shape": shape,
                "z_grad": zt is not None, "propagator": propagator}
        xs = [ray.x, ray.y, ray.dx, ray.dy]
        xs = [v if isinstance(v, torch.Tensor) and v.requires_grad else
              torch.zeros((), device=dev) for v in xs]
        pl = ray.pathlength if isinstance(ray.pathlength, torch.Tensor) and ray.pathlength.requires_grad \
            else torch.zeros((), device=dev, dtype=torch.float64)
        zin = zt if zt is not None else torch.zeros((), device=dev, dtype=torch.float64)
        ox, oy, odx, ody, opl = _TraceFn.apply(spec, *xs, pl, zin, *[p[2] for p in plist])
        zout = spec["zout"]
    else:
        ox, oy, odx, ody, opl, zout, _, _, _ = _fwd_launch(comps, soa, propagator=propagator)
    rs = _reshaper(shape, soa.n)
    out = Ray(x=rs(ox), y=rs(oy), dx=rs(odx), dy=rs(ody), z=zout, pathlength=rs(opl), _one=ray._one)
    return out


def run_component(component: Component, ray: Ray) -> Ray:
    """One component's __call__ on the GPU.  Unlike run_to_end no free-space
    step is applied: the ray must already sit at the component (the reference
    component call does not move the ray)."""
    comps = [component]
    z_s = None
    zz = ray.z
    # The kernel always inserts a propagator; place it at the ray's own z so
    # the inserted distance is exactly 0 (matches components.py semantics).
    import dataclasses as _dc
    if isinstance(zz, torch.Tensor) and zz.dim() > 0 or isinstance(zz, np.ndarray) and zz.ndim > 0:
        raise NotImplementedError("component call on rays with per-ray z")
    z_s = _f(zz)
    if isinstance(component, ThickLens):
        moved = _dc.replace(component, z_po=z_s, z_pi=z_s - (_f(component.z_po) - _f(component.z_pi)))
    elif _dc.is_dataclass(component) and "z" in component.__dataclass_fields__:
        moved = _dc.replace(component, z=z_s)
    else:
        moved = component
    comps = [moved]
    out = run_to_end(ray, comps)
    return out


def passthrough_transform(component):
    """run.py:26-32: wraps one step as ray -> (ray_out, ray_out)."""

    def inner(ray: Ray):
        out = _apply_step(component, ray)
        return out, out

    return inner


def jacobian_transform(component):
    """run.py:35-41: wraps one step as ray -> (ray_out, jac), jac the step's
    Jacobian in the Ray-of-Rays form that ``custom_jacobian_matrix`` reads
    (see ``step_jacobian``)."""

    def inner(ray: Ray):
        return _apply_step(component, ray), step_jacobian(component, ray)

    return inner


def jacobian_and_value(fn, argnums: int = 0, **jac_kwargs):
    """run.py:17-23 for one model step (a component or a Propagator): returns a
    function ray -> (jac, value).  Only the ray argument is differentiated
    (argnums=0)."""
    if argnums != 0:
        raise NotImplementedError("jacobian_and_value differentiates the ray (argnums=0)")

    def inner(ray: Ray):
        return step_jacobian(fn, ray), _apply_step(fn, ray)

    return inner


def _apply_step(step, ray: Ray) -> Ray:
    if isinstance(step, Propagator):
        return step(ray)
    if isinstance(step, Component):
        return run_component(step, ray)
    raise TypeError(f"not a model step: {type(step).__name__}")


def _ray_of_rays(m: np.ndarray) -> Ray:
    """5x5 (rows and columns x, y, dx, dy, _one) -> Ray of Rays; the z and
    pathlength entries are not formed (None)."""
    names = ("x", "y", "dx", "dy", "_one")

    def row(i):
        return Ray(**{n: float(m[i, j]) for j, n in enumerate(names)}, z=None, pathlength=None)

    return Ray(x=row(0), y=row(1), dx=row(2), dy=row(3), z=None, pathlength=None, _one=row(4))


def step_jacobian(step, ray: Ray) -> Ray:
    """Jacobian of one model step (a component call at the ray's plane, or a
    Propagator of fixed distance) about the central ray, as a Ray of Rays:
    ``jac.<out>.<in>`` = d out / d in for out, in in x, y, dx, dy, _one
    (float64, composed on the host from the step's exact matrix, as
    tg_abcd_compose does for the whole model).  The z and pathlength entries,
    which ``custom_jacobian_matrix`` does not read, are None."""
    from .components import Plane
    import dataclasses as _dc
    z0 = _central(ray)[4]
    if isinstance(step, Propagator):
        comps, prop = [Plane(z=z0 + _f(step.distance))], step.propagator
    elif isinstance(step, ThickLens):
        comps, prop = [_dc.replace(step, z_po=z0, z_pi=z0 - (_f(step.z_po) - _f(step.z_pi)))], None
    elif isinstance(step, Component) and _dc.is_dataclass(step) and "z" in step.__dataclass_fields__:
        comps, prop = [_dc.replace(step, z=z0)], None
    else:
        raise TypeError(f"not a model step: {type(step).__name__}")
    return _ray_of_rays(abcd_matrix(ray, comps, prop))


def run_iter(ray: Ray, components: Sequence[Component], transform=passthrough_transform,
             propagator=FreeSpaceParaxial()):
    """run.py:47-82: yields (Propagator, out) then (component, out) per
    element, out = the second value of ``transform(step)(ray)`` (the ray
    itself for passthrough_transform, its Jacobian for jacobian_transform)."""
    for c in _check_model(components):
        d = _f(c.z) - _f(ray.z)
        step = Propagator(d, propagator)
        ray, out = transform(step)(ray)
        yield step, out
        ray, out = transform(c)(ray)
        yield c, out


def _central(ray: Ray):
    r = ray if _ray_scalar_input(ray) else ray[0]
    v = [r.x, r.y, r.dx, r.dy, r.z]
    return [float(np.asarray(a.detach().cpu() if isinstance(a, torch.Tensor) else a).reshape(-1)[0])
            for a in v]


def abcd_matrix(ray: Ray, components: Sequence[Component], propagator=None) -> np.ndarray:
    """float64 5x5 ABCD of the model about a central ray: the reference's
    custom_jacobian_matrix(jax.jacobian(run_to_end)(ray, model))
    (README.md:224-234, utils.py:7-43), composed from component matrices."""
    m, keep = pack_model(components, propagator)
    cen = (C.c_double * 5)(*_central(ray))
    out = (C.c_double * 25)()
    N.check(N.lib().tg_abcd_compose(C.byref(m), cen, out, None), "tg_abcd_compose")
    del keep
    return np.array(out[:], dtype=np.float64).reshape(5, 5)


def solve_model(ray: Ray, model: Sequence[Component], propagator=FreeSpaceParaxial()) -> np.ndarray:
    """run.py:150-179: per-step 5x5 matrices, shape (2*n_components, 5, 5)."""
    comps = _check_model(model)
    m, keep = pack_model(comps, propagator)
    cen = (C.c_double * 5)(*_central(ray))
    out = (C.c_double * 25)()
    steps = (C.c_double * (50 * max(1, len(comps))))()
    N.check(N.lib().tg_abcd_compose(C.byref(m), cen, out, steps), "tg_abcd_compose")
    del keep
    return np.array(steps[:50 * len(comps)], dtype=np.float64).reshape(-1, 5, 5)


def calculate_derivatives(ray: Ray, model: Sequence[Component], order: int):
    """run.py:118-147 for order 1: [the Jacobian of run_to_end with respect to
    the ray] as a Ray of Rays (x, y, dx, dy, _one entries, float64, about the
    central ray).  The adjoint kernels are first order: order > 1 raises."""
    if order < 1:
        return []
    if order > 1:
        raise NotImplementedError("derivatives beyond the first are not formed on the GPU")
    return [_ray_of_rays(abcd_matrix(ray, model))]


# ------------------------------------------------------------- run_with_grads
_RAY_VARS = ("x", "y", "dx", "dy", "z", "pathlength")
_OUT_FIELDS = ("x", "y", "dx", "dy", "pathlength")


class _Ident:
    """Dictionary key part for an unhashable root (a Ray holding arrays):
    hashed and compared by identity."""

    def __init__(self, obj):
        self.obj = obj

    def __hash__(self):
        return id(self.obj)

    def __eq__(self, other):
        return self.obj is (other.obj if isinstance(other, _Ident) else other)

    def __repr__(self):
        return f"<{type(self.obj).__name__} at {id(self.obj):#x}>"


def _key(root, *path):
    try:
        hash(root)
        return (root,) + path
    except TypeError:
        return (_Ident(root),) + path


def _param_paths(comp, path) -> list:
    """Parameter names (as param_gradient spells them) under a path into a
    component: a field, descan_error (all its coefficients) or one of them."""
    from .components import DescanError
    if len(path) == 1 and path[0] == "descan_error" and isinstance(getattr(comp, "descan_error", None),
                                                                   DescanError):
        return ["descan_error." + f for f in DescanError._fields]
    if len(path) == 2 and path[0] == "descan_error" and path[1] in getattr(DescanError, "_fields", ()):
        return ["descan_error." + path[1]]
    fields = getattr(comp, "__dataclass_fields__", {})
    if len(path) == 1 and (path[0] in fields or (isinstance(comp, ThickLens) and path[0] in ("z_po", "z_pi"))):
        return [path[0]]
    return []


def _with_param(comp, name, t):
    import dataclasses as _dc
    if name.startswith("descan_error."):
        dn = name.split(".", 1)[1]
        return _dc.replace(comp, descan_error=comp.descan_error._replace(**{dn: t}))
    return _dc.replace(comp, **{name: t})


def run_with_grads(input_ray: Ray, model: Sequence[Component], grad_vars):
    """run.py:182-267: run the model and return (value, grads), grads mapping
    each selected variable's path (root object, keys...) to a Ray of
    d(output field)/d(variable).

    ``grad_vars``: the input ray itself (all of x, y, dx, dy, z, pathlength),
    ``input_ray.params.<field>``, or ``component.params.<field>`` (also
    ``descanner.params.descan_error[.<coefficient>]``) for components of
    ``model``; an unknown path raises RuntimeError, as the reference does.
    Shapes follow jax.jacobian: a per-ray input field gives (N, N) blocks
    (diagonal: rays are independent), a shared scalar gives (N,).

    The derivatives come from the adjoint kernel (tg_trace_vjp) through
    torch.autograd: one pass per output field for per-ray inputs, and one
    pass per output field and ray for shared parameters (the kernel sums a
    parameter's sensitivity over rays).  d/d _one is not formed."""
    from .ray import is_uniform
    from .tree_utils import PathBuilder
    import dataclasses as _dc
    comps = list(_check_model(model))
    ray_sel, comp_sel = [], []  # (key, field) / (key, component index, parameter name)
    for var in grad_vars:
        before = len(ray_sel) + len(comp_sel)
        if var is input_ray:
            ray_sel += [(_key(input_ray, f), f) for f in _RAY_VARS]
        elif isinstance(var, PathBuilder):
            root, path = var._resolve_root(), var._build()[1:]
            if root is input_ray:
                if path == ("_one",):
                    raise NotImplementedError("derivatives with respect to _one are not formed")
                if len(path) == 1 and path[0] in _RAY_VARS:
                    ray_sel.append((_key(input_ray, *path), path[0]))
            else:
                for i, c in enumerate(comps):
                    if c is root:
                        comp_sel += [(_key(root, *tuple(nm.split("."))), i, nm) for nm in _param_paths(c, path)]
                        break
        if len(ray_sel) + len(comp_sel) == before:
            raise RuntimeError(f"Cannot find {var!r} in parameters")

    dev = _device()
    shape = _in_shape(input_ray)
    n = int(np.prod(shape)) if shape else 1
    kw = {f.name: getattr(input_ray, f.name) for f in _dc.fields(input_ray)}
    per_ray, shared = {}, {}  # leaf tensors
    for _, f in ray_sel:
        if f in per_ray or f in shared or f == "pathlength":
            continue  # pathlength enters the output pathlength only: d = 1, done analytically
        v = kw[f]
        if f == "z":
            if not is_uniform(v):
                raise NotImplementedError("d/dz needs one z for all rays")
            t = torch.tensor(_f(v), dtype=torch.float64, requires_grad=True)
            shared["z"] = t
        else:
            src = v.detach() if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v, np.float32))
            t = src.to(device=dev, dtype=torch.float32).expand(shape).contiguous().requires_grad_(True)
            per_ray[f] = t
        kw[f] = t
    cm = list(comps)
    for _, i, name in comp_sel:
        if (i, name) in shared:
            continue
        cur = getattr(cm[i].descan_error, name.split(".", 1)[1]) if name.startswith("descan_error.") \
            else getattr(cm[i], name)
        t = torch.tensor(_f(cur), dtype=torch.float64, requires_grad=True)
        shared[(i, name)] = t
        cm[i] = _with_param(cm[i], name, t)
    with torch.enable_grad():
        out = run_to_end(type(input_ray)(**kw) if type(input_ray) is Ray else Ray(
            **{k: kw[k] for k in ("x", "y", "dx", "dy", "z", "pathlength", "_one")}), cm)
    outs = {k: getattr(out, k) for k in _OUT_FIELDS}
    f64 = dict(dtype=torch.float64, device=dev)
    d = {}  # (var id, out field) -> tensor shaped like the output field
    pr_names = list(per_ray)
    sh_keys = list(shared)
    for k in _OUT_FIELDS:
        o = outs[k]
        if pr_names:
            g = torch.autograd.grad(o, [per_ray[f] for f in pr_names], grad_outputs=torch.ones_like(o),
                                    retain_graph=True, allow_unused=True)
            for f, gv in zip(pr_names, g):
                d[(f, k)] = torch.zeros(shape, **f64) if gv is None else gv.to(torch.float64)
        if sh_keys:
            cols = {s: torch.zeros(shape, **f64) for s in sh_keys}
            for i in range(n):
                seed = torch.zeros_like(o)
                if shape:
                    seed[i] = 1
                else:
                    seed.fill_(1)
                g = torch.autograd.grad(o, [shared[s] for s in sh_keys], grad_outputs=seed,
                                        retain_graph=True, allow_unused=True)
                for s, gv in zip(sh_keys, g):
                    if gv is not None:
                        if shape:
                            cols[s][i] = gv.to(torch.float64).to(dev)
                        else:
                            cols[s] = gv.to(torch.float64).to(dev).reshape(())
            for s in sh_keys:
                d[(s, k)] = cols[s]
    last = len(comps) - 1
    z_var = (last, "z_pi") if isinstance(comps[-1], ThickLens) else (last, "z")

    def jac(var, field_shared: bool):
        """Ray of d(out)/d(var); per-ray inputs become (N, N) diagonal blocks."""
        def blk(v):
            return torch.diag_embed(v) if (shape and not field_shared) else v
        fields = {}
        for k in _OUT_FIELDS:
            if var == "pathlength":
                v = torch.ones(shape, **f64) if k == "pathlength" else torch.zeros(shape, **f64)
            else:
                v = d[(var, k)]
            fields[k] = blk(v)
        fields["z"] = blk(torch.ones(shape, **f64) if var == z_var else torch.zeros(shape, **f64))
        fields["_one"] = blk(torch.zeros(shape, **f64))
        return Ray(**fields)

    grads = {}
    for key, f in ray_sel:
        shared_field = f == "z" or (shape and not _is_per_ray(getattr(input_ray, f), n))
        # a scalar field given for vector rays is shared: its column is the per-ray derivative
        grads[key] = jac(f, bool(shared_field))
    for key, i, name in comp_sel:
        grads[key] = jac((i, name), True)
    value = Ray(**{k: (v.detach() if isinstance(v, torch.Tensor) else v)
                   for k, v in ((f.name, getattr(out, f.name)) for f in _dc.fields(out))})
    return value, grads


def _is_per_ray(v, n) -> bool:
    return isinstance(v, (torch.Tensor, np.ndarray)) and v.ndim > 0 and int(np.prod(v.shape)) == n and n > 0


# ------------------------------------------------------------------ binning

def bin_pixels(grid: Grid, x, y):
    """Bit-exact metres->pixels on the GPU (grid.py:120-153)."""
    dev = _device()
    xt = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, dtype=np.float32))
    yt = y if isinstance(y, torch.Tensor) else torch.as_tensor(np.asarray(y, dtype=np.float32))
    shape = tuple(xt.shape)
    n = max(xt.numel(), yt.numel())
    xs = as_f32(xt, n, dev)
    ys = as_f32(yt, n, dev)
    py = torch.empty(n, dtype=torch.int32, device=dev)
    px = torch.empty(n, dtype=torch.int32, device=dev)
    g = grid._tg_grid()
    N.check(N.lib().tg_bin(n, N.ptr(xs), N.ptr(ys), None, C.byref(g), N.ptr(py), N.ptr(px),
                           None, 0, N.stream_ptr()), "tg_bin")
    from . import PixelsYX
    return PixelsYX(y=py.reshape(shape), x=px.reshape(shape))


def image_from(grid: Grid, ray, acc=None):
    """grid.py:231-280 on the GPU."""
    dev = _device()
    h, w = int(grid.shape[0]), int(grid.shape[1])
    if acc is None:
        acc = torch.zeros((h, w), dtype=torch.int64, device=dev)
    if tuple(acc.shape) != (h, w):
        raise ValueError(f"accumulator shape {tuple(acc.shape)} != grid shape {(h, w)}")
    if acc.dtype not in (torch.int32, torch.int64) or not acc.is_cuda or not acc.is_contiguous():
        raise TypeError("accumulator must be a contiguous int32/int64 CUDA tensor")
    lib = N.lib()
    if isinstance(ray, Ray):
        n = ray.size
        xs = as_f32(ray.x, n, dev)
        ys = as_f32(ray.y, n, dev)
        g = grid._tg_grid()
        ws_bytes = lib.tg_hist_workspace(n, h, w)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev) if ws_bytes else None
        N.check(lib.tg_bin_image(n, N.ptr(xs), N.ptr(ys), None, C.byref(g), None, None,
                                 N.ptr(acc), 1 if acc.dtype == torch.int64 else 0,
                                 N.ptr(ws), ws_bytes, N.stream_ptr()), "tg_bin_image")
        return acc
    # PixelsYX input: integer indices already computed (int32 kept, others as int64)
    py, px = ray
    py = torch.as_tensor(py, device=dev).reshape(-1)
    px = torch.as_tensor(px, device=dev).reshape(-1)
    if py.numel() != px.numel():
        raise ValueError("pixel index arrays differ in length")
    idt = torch.int32 if (py.dtype == torch.int32 and px.dtype == torch.int32) else torch.int64
    py, px = py.to(idt).contiguous(), px.to(idt).contiguous()
    n = py.numel()
    ws_bytes = lib.tg_hist_workspace(n, h, w)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev) if ws_bytes else None
    N.check(lib.tg_hist_pixels(n, N.ptr(py), N.ptr(px), 1 if idt == torch.int64 else 0, h, w,
                               N.ptr(acc), 1 if acc.dtype == torch.int64 else 0, N.ptr(ws), ws_bytes,
                               N.stream_ptr()), "tg_hist_pixels")
    return acc


def trace_to_image(ray: Ray, components: Sequence[Component], detector: Grid | None = None,
                   acc: torch.Tensor | None = None, want_pixels: bool = True):
    """Fused run_to_end + Detector.metres_to_pixels + Detector.into_image in a
    single kernel pass.  Returns (ray_out, PixelsYX or None, image)."""
    comps = _check_model(components)
    if detector is None:
        detector = comps[-1]
    if not isinstance(detector, Grid):
        raise ValueError("trace_to_image needs a Detector/ScanGrid")
    dev = _device()
    soa = _Soa(ray, dev)
    h, w = int(detector.shape[0]), int(detector.shape[1])
    if acc is None:
        acc = torch.zeros((h, w), dtype=torch.int64, device=dev)
    ox, oy, odx, ody, opl, zout, oamp, py, px = _fwd_launch(comps, soa, detector, want_pixels, acc)
    shape = _in_shape(ray)
    rs = _reshaper(shape, soa.n)
    out = Ray(x=rs(ox), y=rs(oy), dx=rs(odx), dy=rs(ody), z=zout, pathlength=rs(opl), _one=ray._one)
    from . import PixelsYX
    pix = PixelsYX(y=rs(py), x=rs(px)) if want_pixels else None
    return out, pix, acc


def _reshaper(shape, n):
    """Reshape to the input's shape, skipping the no-op case (vector input)."""
    if shape == (n,):
        return lambda t: t
    return lambda t: t.reshape(shape)


class TracePlan:
    """A compiled trace for repeated launches on the same device buffers.

    Packs the model once, allocates the outputs once and keeps the C-ABI
    structures, so ``run()`` is a single C call (no Python allocation) and
    ``capture()`` records it as a CUDA graph.  ``x, y, dx, dy`` are float32
    CUDA tensors of equal length whose contents may change between runs;
    ``z`` and ``pathlength`` are uniform inputs.  With a detector the launch
    also bins the rays and adds them to ``self.image``.
    """

    def __init__(self, components, x, y, dx, dy, z=0.0, pathlength=0.0, detector: Grid | None = None,
                 pixels: bool = False, hist_dtype=torch.int64, propagator=None):
        N.require_cuda(x)
        self.comps = _check_model(components)
        for t in (x, y, dx, dy):
            if t.dtype != torch.float32 or not t.is_contiguous() or t.numel() != x.numel():
                raise ValueError("x, y, dx, dy must be contiguous float32 tensors of equal length")
        self.n = x.numel()
        self.inputs = (x, y, dx, dy)
        dev = x.device
        self.out = tuple(torch.empty(self.n, dtype=torch.float32, device=dev) for _ in range(4))
        self.pathlength = torch.empty(self.n, dtype=torch.float64, device=dev)
        self._m, self._keep = pack_model(self.comps, propagator)
        self._in = _rays_struct(self.n, x, y, dx, dy, None, float(z), None, float(pathlength))
        self._o = _rays_struct(self.n, *self.out, None, 0.0, self.pathlength, 0.0)
        self._zout = C.c_double(0.0)
        self.detector = detector
        self.image = None
        self.pix = None
        self._g = None
        self._ws, self._ws_bytes = None, 0
        if detector is not None:
            self._g = detector._tg_grid()
            h, w = int(detector.shape[0]), int(detector.shape[1])
            self.image = torch.zeros((h, w), dtype=hist_dtype, device=dev)
            ws_bytes = N.lib().tg_trace_image_workspace(self.n, C.byref(self._g))
            self._ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev) if ws_bytes else None
            self._ws_bytes = ws_bytes
            if pixels:
                self.pix = (torch.empty(self.n, dtype=torch.int32, device=dev),
                            torch.empty(self.n, dtype=torch.int32, device=dev))
        self._lib = N.lib()
        self.graph = None

    def run(self):
        pix = self.pix or (None, None)
        st = self._lib.tg_trace_image(C.byref(self._m), C.byref(self._in), C.byref(self._o),
                                      C.byref(self._zout), C.byref(self._g) if self._g is not None else None,
                                      N.ptr(pix[0]), N.ptr(pix[1]), N.ptr(self.image),
                                      1 if (self.image is not None and self.image.dtype == torch.int64) else 0,
                                      N.ptr(self._ws), self._ws_bytes, N.stream_ptr())
        N.check(st, "tg_trace_image")
        return self

    def capture(self):
        """Record one run as a CUDA graph (``self.graph.replay()``)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def ray(self) -> Ray:
        return Ray(x=self.out[0], y=self.out[1], dx=self.out[2], dy=self.out[3], z=self._zout.value,
                   pathlength=self.pathlength)
