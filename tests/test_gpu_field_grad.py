"""Adjoint of the beamlet field (tg_field_vjp behind make_gaussian_image /
evaluate_gaussian_input_image under torch.autograd) against central finite
differences of the float64 oracle (oracle/field.py, exact k*pl reduction).

Loss L = Re sum conj(T) F for a seeded complex image T (its gradient with
respect to F is T; a loss without a large constant keeps the float64
differences of the oracle well above their rounding).  Bounds (normwise over
each group of gradients): x, y, dx, dy, focal length, detector z and the
amplitudes <= 1e-4 relative (finite-difference steps where the float64
differences have converged); the pathlength gradient equals k times the
gradient with respect to the amplitude's phase (F depends on pl only through
exp(i k pl)) to 1e-6."""
import numpy as np
import pytest
import torch

import oracle.field as OF
from conftest import normwise_err

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _rays_t(d, dev, req=True):
    """GaussianRay with differentiable float64 / complex64 device tensors."""
    import temgymcore_gb300 as t
    f = lambda k: torch.tensor(np.asarray(d[k], np.float64), device=dev, requires_grad=req)  # noqa: E731
    amp = torch.tensor(np.asarray(d["amplitude"], np.complex64), device=dev, requires_grad=req)
    return t.GaussianRay(x=f("x"), y=f("y"), dx=f("dx"), dy=f("dy"), z=d["z"], pathlength=f("pathlength"),
                         amplitude=amp, waist_xy=d["waist_xy"], radii_of_curv=d["radii_of_curv"],
                         wavelength=d["wavelength"], theta=d["theta"])


def _target(shape, seed, scale):
    rng = np.random.default_rng(seed)
    return (scale * (rng.normal(size=shape) + 1j * rng.normal(size=shape))).astype(np.complex128)


def _oracle_loss(rays, model, target):
    F = OF.make_gaussian_image(rays, model, phase_mode="exact")
    return float(np.real(np.sum(np.conj(target) * F)))


def _loss_t(F, T):
    return (torch.conj(T) * F).real.sum()


def _fd(fn, v, h):
    return (fn(v + h) - fn(v - h)) / (2 * h)


@pytest.mark.parametrize("astig", [True, False])
def test_field_gradients_against_oracle_fd(cuda, astig):
    from temgymcore_gb300 import make_gaussian_image
    from temgymcore_gb300.components import Detector, Lens
    from temgymcore_gb300.workloads import beamlet_field
    w = beamlet_field(seed=2, n_beams=48, det_shape=(40, 56), det_px=3e-5, astigmatic=astig)
    rays_np = w["rays"]
    # a lens of 0.4 m at 0.5 m: the detector at 1.0 m sits 0.1 m past the
    # back focal plane, so the focal length and the detector z both matter
    spec = [{"kind": "lens", "z": 0.5, "focal_length": 0.4},
            {"kind": "detector", "z": 1.0, "pixel_size": (3e-5, 3e-5), "shape": (40, 56)}]
    f_t = torch.tensor(0.4, dtype=torch.float64, requires_grad=True)
    z_t = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    model = [Lens(z=0.5, focal_length=f_t), Detector(z=z_t, pixel_size=(3e-5, 3e-5), shape=(40, 56))]
    F0 = OF.make_gaussian_image(rays_np, spec, phase_mode="exact")
    T = _target(F0.shape, 5, 0.5 * np.abs(F0).max())
    r = _rays_t(rays_np, cuda)
    F = make_gaussian_image(r, model)
    _loss_t(F, torch.tensor(T.astype(np.complex64), device=cuda)).backward()
    assert normwise_err(F.detach().cpu().numpy(), F0) <= 1e-5
    beams = [0, 7, 23, 41]
    # central ray positions and slopes (steps where the float64 differences
    # have converged: the loss is 1e5 times less sensitive to the slopes)
    for key, h in (("x", 1e-13), ("y", 1e-13), ("dx", 1e-10), ("dy", 1e-10)):
        ref, got = [], []
        for b in beams:
            def fn(v, b=b, key=key):
                d = dict(rays_np)
                a = np.array(d[key], np.float64)
                a[b] = v
                d[key] = a
                return _oracle_loss(d, spec, T)
            ref.append(_fd(fn, float(rays_np[key][b]), h))
            got.append(float(getattr(r, key).grad[b]))
        assert normwise_err(got, ref) <= TOL, (key, got, ref)
    # amplitudes (the loss is quadratic in them: central differences are exact)
    ref, got = [], []
    for b in beams:
        for part in (1.0, 1j):
            def fn(v, b=b, part=part):
                d = dict(rays_np)
                a = np.array(d["amplitude"], np.complex128)
                a[b] = a[b] + v * part
                d["amplitude"] = a
                return _oracle_loss(d, spec, T)
            ref.append(_fd(fn, 0.0, 1e-3))
        g = complex(r.amplitude.grad[b])
        got += [g.real, g.imag]
    assert normwise_err(got, ref) <= TOL
    # model parameters: the lens focal length and the detector's z
    def f_loss(v):
        s2 = [dict(c) for c in spec]
        s2[0]["focal_length"] = v
        return _oracle_loss(rays_np, s2, T)

    def z_loss(v):
        s2 = [dict(c) for c in spec]
        s2[1]["z"] = v
        return _oracle_loss(rays_np, s2, T)
    ref = [_fd(f_loss, 0.4, 1e-10), _fd(z_loss, 1.0, 1e-9)]
    got = [float(f_t.grad), float(z_t.grad)]
    assert normwise_err(got, ref) <= TOL, (got, ref)
    # pathlength: F depends on pl through exp(i k pl) only
    k = 2 * np.pi / rays_np["wavelength"]
    a = r.amplitude.detach().cpu().numpy().astype(np.complex128)
    ga = r.amplitude.grad.cpu().numpy().astype(np.complex128)
    dphi = np.real(np.conj(ga) * 1j * a)
    assert normwise_err(r.pathlength.grad.cpu().numpy(), k * dphi) <= 1e-6


def test_input_field_gradients_against_oracle_fd(cuda):
    from temgymcore_gb300 import evaluate_gaussian_input_image
    from temgymcore_gb300.workloads import build_model, input_field
    w = input_field(seed=3, n_beams=40, grid_shape=(36, 44), px=1e-5)
    rays_np, grid_spec = w["rays"], w["grid"]
    grid = build_model([grid_spec])[0]
    F0 = OF.evaluate_gaussian_input_image(rays_np, grid_spec, phase_mode="exact")
    T = _target(F0.shape, 6, 0.5 * np.abs(F0).max())
    r = _rays_t(rays_np, cuda)
    F = evaluate_gaussian_input_image(r, grid)
    _loss_t(F, torch.tensor(T.astype(np.complex64), device=cuda)).backward()
    beams = [1, 9, 30]
    for key, h in (("x", 1e-9), ("y", 1e-9), ("dx", 1e-7), ("dy", 1e-7)):
        ref, got = [], []
        for b in beams:
            def fn(v, b=b, key=key):
                d = dict(rays_np)
                a = np.array(d[key], np.float64)
                a[b] = v
                d[key] = a
                return float(np.real(np.sum(np.conj(T) * OF.evaluate_gaussian_input_image(
                    d, grid_spec, phase_mode="exact"))))
            ref.append(_fd(fn, float(rays_np[key][b]), h))
            got.append(float(getattr(r, key).grad[b]))
        assert normwise_err(got, ref) <= TOL, (key, got, ref)


def test_field_vjp_full_size_directional_derivative(cuda):
    """16,384 beams on 512 x 512 pixels (the benchmark's beamlet workload):
    the adjoint's gradient along random directions of the central rays against
    central differences of the all-float64 field kernel on the GPU."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    w = beamlet_field(seed=0)
    comps = build_model(w["model"])
    plan = t.FieldPlan(gaussian_rays(w["rays"]), comps, method="fp64")
    F = plan.evaluate("fp64").clone()
    T = torch.tensor(_target(plan.shape, 8, 0.5 * float(F.abs().max())).astype(np.complex64), device=cuda)
    r = plan.vjp(T)  # L = Re sum conj(T) F: its gradient image is T
    rng = np.random.default_rng(4)
    for key in ("x", "dx"):
        v = rng.normal(size=16384)
        # the same phase change for both: the field is ~1e6 times less
        # sensitive to the slopes than to the positions at the focal plane
        h = 1e-13 if key == "x" else 1e-7

        def L(sign):
            d = dict(w["rays"])
            d[key] = np.asarray(d[key], np.float64) + sign * h * v
            p = t.FieldPlan(gaussian_rays(d), comps, method="fp64")
            Fp = p.evaluate("fp64").to(torch.complex128)
            return float((torch.conj(T.to(torch.complex128)) * Fp).real.sum())
        ref = (L(1) - L(-1)) / (2 * h)
        got = float((r[key].cpu().numpy() * v).sum())
        assert abs(got - ref) <= 1e-3 * abs(ref), (key, got, ref)


@pytest.mark.parametrize("full", [False, True])
def test_separable_moments_on_tensor_cores_match_direct(cuda, full):
    """Separable beams: the adjoint's per-beam moments from the tensor-core
    GEMM (X_a = conj(G) (U dc^a)^T, then the rows with V dr^k) against the
    direct pass over beams x pixels: every gradient group agrees to 1e-4
    normwise (split-BF16 operands, as the separable forward), on a small
    ragged detector and on the full 16,384-beam, 512 x 512 workload."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    w = beamlet_field(seed=0) if full else beamlet_field(seed=2, n_beams=300, det_shape=(45, 70), det_px=3e-5)
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    assert plan.separable and plan.method == "separable"
    F = plan.evaluate("separable").clone()
    T = torch.tensor(_target(plan.shape, 11, 0.5 * float(F.abs().max())).astype(np.complex64), device=cuda)
    a = plan.vjp(T, method="separable")
    b = plan.vjp(T, method="direct")
    def real(x):
        return (torch.view_as_real(x) if x.is_complex() else x).cpu().numpy()
    for k in ("amplitude", "pathlength", "x", "y", "dx", "dy", "raw"):
        u, v = real(a[k]), real(b[k])
        assert normwise_err(u, v) <= 1e-4, (k, normwise_err(u, v))
    assert t._native.error_word() == 0


def test_separable_adjoint_flags_astigmatic_beams(cuda):
    """The tensor-core moments assume separable beams; given astigmatic ones
    the call reports TG_EW_NONSEPARABLE in the error word (as the separable
    forward does)."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    w = beamlet_field(seed=2, n_beams=64, det_shape=(32, 40), det_px=3e-5, astigmatic=True)
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    assert not plan.separable
    t._native.error_word()
    T = torch.ones(plan.shape, dtype=torch.complex64, device=cuda)
    plan.vjp(T, method="separable")
    assert t._native.error_word() & 0x10
    plan.vjp(T)  # the plan's own (direct) method
    assert t._native.error_word() == 0


def test_field_gradients_deep_model_many_directions(cuda):
    """A 15-component chain (deflectors, rotators, lenses): 38 derivative
    directions, so the adjoint's chain rule runs several step groups and two
    launches (32 directions a launch).  Parameters from different groups and
    from both launches against central differences of the float64 oracle."""
    from temgymcore_gb300 import make_gaussian_image
    from temgymcore_gb300.components import Deflector, Detector, Lens, Rotator
    from temgymcore_gb300.workloads import beamlet_field
    shape, px = (32, 40), 3e-5
    w = beamlet_field(seed=3, n_beams=32, det_shape=shape, det_px=px)
    rays_np = w["rays"]
    spec = []
    for i in range(15):
        z = 0.05 + 0.06 * i
        kind = ("deflector", "rotator", "lens")[i % 3]
        if kind == "deflector":
            spec.append({"kind": "deflector", "z": z, "def_x": 2e-7 * (i + 1), "def_y": -1e-7 * (i + 2)})
        elif kind == "rotator":
            spec.append({"kind": "rotator", "z": z, "angle": 7.0 * (i + 1)})
        else:
            spec.append({"kind": "lens", "z": z, "focal_length": 0.6 + 0.1 * i})
    spec.append({"kind": "detector", "z": 1.0, "pixel_size": (px, px), "shape": shape})
    # differentiable parameters: the last deflector's def_y (its directions
    # fall in the second launch), a rotator's angle, a lens's focal length
    # and the detector's z
    t_defy = torch.tensor(spec[12]["def_y"], dtype=torch.float64, requires_grad=True)
    t_ang = torch.tensor(spec[4]["angle"], dtype=torch.float64, requires_grad=True)
    t_f = torch.tensor(spec[8]["focal_length"], dtype=torch.float64, requires_grad=True)
    t_z = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    model = []
    for i, c in enumerate(spec):
        k = c["kind"]
        if k == "deflector":
            model.append(Deflector(z=c["z"], def_x=c["def_x"], def_y=t_defy if i == 12 else c["def_y"]))
        elif k == "rotator":
            model.append(Rotator(z=c["z"], angle=t_ang if i == 4 else c["angle"]))
        elif k == "lens":
            model.append(Lens(z=c["z"], focal_length=t_f if i == 8 else c["focal_length"]))
        else:
            model.append(Detector(z=t_z, pixel_size=(px, px), shape=shape))
    F0 = OF.make_gaussian_image(rays_np, spec, phase_mode="exact")
    T = _target(F0.shape, 11, 0.5 * np.abs(F0).max())
    F = make_gaussian_image(_rays_t(rays_np, cuda, req=False), model)
    assert normwise_err(F.detach().cpu().numpy(), F0) <= 1e-5
    _loss_t(F, torch.tensor(T.astype(np.complex64), device=cuda)).backward()

    def loss_at(i, key, v):
        s2 = [dict(c) for c in spec]
        s2[i][key] = v
        return _oracle_loss(rays_np, s2, T)
    ref = [_fd(lambda v: loss_at(12, "def_y", v), spec[12]["def_y"], 1e-12),
           _fd(lambda v: loss_at(4, "angle", v), spec[4]["angle"], 1e-7),
           _fd(lambda v: loss_at(8, "focal_length", v), spec[8]["focal_length"], 1e-10),
           _fd(lambda v: loss_at(15, "z", v), 1.0, 1e-9)]
    got = [float(t_defy.grad), float(t_ang.grad), float(t_f.grad), float(t_z.grad)]
    # measured: def_y 9e-8, angle 3.4e-5 (its differences carry ~1e-5 of
    # noise: the spiral bundle is nearly symmetric under rotation), focal
    # length 7.8e-6, z 2.3e-6
    errs = {name: abs(g - r) / abs(r) for g, r, name in zip(got, ref, ("def_y", "angle", "focal_length", "z"))}
    for name, e in errs.items():
        assert e <= TOL, (name, errs, got, ref)
