"""AberratedLensKrivanek on the GPU against the float64 oracle (the
reference's polar-form series, components.py:177-215 and
aberrations.py:42-108): fused trace + bit-exact binning, the 4D-STEM scan
kernel, and the beamlet field prepared through the lens (its Jacobian enters
each beam's ABCD).  Coordinates <= 2e-6 normwise (float32 ray state with the
aberration polynomial evaluated in float32); pixels and histograms bit-exact
given the same float32 coordinates; field tolerances as for the other
beamlet-field tests.  The adjoint and batched paths reject the component."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from oracle import field as OF
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu

NAMES = oracle.rays._KRIV


def _coeffs(rng, f, alpha):
    c = {}
    for n in NAMES:
        if n.startswith("phi"):
            c[n] = float(rng.uniform(-np.pi, np.pi))
        else:
            order = int(n[1])
            c[n] = float(rng.normal(0.0, 0.1 * f / alpha ** (order - 1) / (order + 1)))
    return c


def np_(t):
    return t.detach().cpu().numpy()


def test_trace_and_binning_through_aberrated_lens(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(0)
    n = 65536
    x = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    y = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    dx = rng.normal(0, 1e-3, n).astype(np.float32)
    dy = rng.normal(0, 1e-3, n).astype(np.float32)
    spec = [{"kind": "lens", "z": 0.2, "focal_length": 0.5},
            {"kind": "aberrated_lens", "z": 0.5, "focal_length": 0.2, "coeffs": _coeffs(rng, 0.2, 3e-3)},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (256, 256)}]
    ray = t.Ray(x=torch.tensor(x, device=cuda), y=torch.tensor(y, device=cuda),
                dx=torch.tensor(dx, device=cuda), dy=torch.tensor(dy, device=cuda), z=0.0, pathlength=0.0)
    out, pix, img = t.trace_to_image(ray, build_model(spec))
    ref = oracle.run_to_end(ORay.from_f32(x, y, dx, dy, 0.0, 0.0), spec)
    for k in ("x", "y", "dx", "dy"):
        assert normwise_err(np_(getattr(out, k)), getattr(ref, k)) <= 2e-6, k
    assert normwise_err(np_(out.pathlength), ref.pathlength) <= 1e-9
    # the aberration moved the rays (not a no-op)
    plain = oracle.run_to_end(ORay.from_f32(x, y, dx, dy, 0.0, 0.0),
                              [spec[0], {"kind": "lens", "z": 0.5, "focal_length": 0.2}, spec[2]])
    assert normwise_err(ref.x, plain.x) > 1e-3
    g = {"pixel_size": (1e-5, 1e-5), "shape": (256, 256)}
    py, px = oracle.metres_to_pixels(g, np_(out.x).astype(np.float64), np_(out.y).astype(np.float64))
    assert np.array_equal(np_(pix.y), py) and np.array_equal(np_(pix.x), px)
    assert np.array_equal(np_(img), oracle.into_image(g, py, px))
    # single-component call and run_to_end agree with the fused call
    out2 = t.run_to_end(ray, build_model(spec))
    assert torch.equal(out2.x, out.x) and torch.equal(out2.dy, out.dy)
    assert t._native.error_word() == 0


def test_scan_through_aberrated_lens(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_4d, stem_model, stem_probe_model
    rng = np.random.default_rng(1)
    w = stem_4d(seed=2, scan=(4, 3), rays_per_probe=1024)
    ab = {"kind": "aberrated_lens", "z": 0.03, "focal_length": 0.05, "coeffs": _coeffs(rng, 0.05, 2e-3)}
    model = stem_model(w)
    model.insert(4, t.AberratedLensKrivanek(z=ab["z"], focal_length=ab["focal_length"], coeffs=ab["coeffs"]))
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                z=0.0, pathlength=0.0)
    imgs, xy = t.scan_images(ray, model, return_xy=True)
    pos = t.scan_positions(model[1])
    g = {k: w["detector"][k] for k in ("pixel_size", "shape")}
    for p in range(imgs.shape[0]):
        spec = stem_probe_model(w, *pos[p])
        spec.insert(4, ab)
        ref = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], w["z"], 0.0), spec)
        gx, gy = np_(xy[p, 0]), np_(xy[p, 1])
        assert normwise_err(gx, ref.x) <= 2e-6 and normwise_err(gy, ref.y) <= 2e-6, p
        py, px = oracle.metres_to_pixels(g, gx.astype(np.float64), gy.astype(np.float64))
        assert np.array_equal(np_(imgs[p]), oracle.into_image(g, py, px).astype(np.int32)), p
    assert t._native.error_word() == 0


def _cmp_field(got, ref, tol, ptol=1e-4):
    got = got.astype(np.complex128)
    e = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert e <= tol, e
    bright = np.abs(ref) > 0.25 * np.max(np.abs(ref))
    assert np.abs(np.angle(got[bright] * np.conj(ref[bright]))).max() <= ptol


def test_field_through_aberrated_lens(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    rng = np.random.default_rng(2)
    spec = [{"kind": "aberrated_lens", "z": 0.3, "focal_length": 0.4, "coeffs": _coeffs(rng, 0.4, 1.5e-3)},
            {"kind": "detector", "z": 0.7, "pixel_size": (2e-5, 2e-5), "shape": (48, 64)}]
    nb = 24
    r = {"x": rng.uniform(-3e-4, 3e-4, nb), "y": rng.uniform(-3e-4, 3e-4, nb),
         "dx": rng.normal(0, 1e-3, nb), "dy": rng.normal(0, 1e-3, nb), "z": 0.0,
         "pathlength": rng.uniform(0.5, 1.0, nb),
         "amplitude": (rng.uniform(0.5, 1, nb) * np.exp(2j * np.pi * rng.uniform(size=nb))).astype(np.complex64),
         "waist_xy": np.full((nb, 2), 1.5e-4), "radii_of_curv": np.full((nb, 2), np.inf),
         "wavelength": 500e-9, "theta": np.zeros(nb)}
    ref = OF.make_gaussian_image(r, spec)
    plan = t.FieldPlan(gaussian_rays(r), build_model(spec))
    _cmp_field(np_(plan.evaluate("fp64")), ref, 5e-7, 5e-7)
    _cmp_field(np_(plan.evaluate("direct")), ref, 1e-4)
    assert t._native.error_word() == 0


def test_adjoint_and_batched_reject_aberrated_lens(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace
    model = [t.AberratedLensKrivanek(z=0.5, focal_length=0.2, coeffs={"C30": 1e3}),
             t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(8, 8))]
    x = torch.zeros(4, device=cuda, requires_grad=True)
    out = t.run_to_end(t.Ray(x=x, y=torch.zeros(4, device=cuda), dx=torch.zeros(4, device=cuda),
                             dy=torch.zeros(4, device=cuda), z=0.0, pathlength=0.0), model)
    with pytest.raises(RuntimeError):
        out.x.sum().backward()
    with pytest.raises(RuntimeError):
        BatchedTrace([model], [16])
    assert N.error_word() == 0
