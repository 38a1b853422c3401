"""AberratedLensKrivanek on the GPU against the float64 oracle (the
reference's polar-form series, components.py:177-215 and
aberrations.py:42-108): fused trace + bit-exact binning, the 4D-STEM scan
kernel, and the beamlet field prepared through the lens (its Jacobian enters
each beam's ABCD).  Coordinates <= 2e-6 normwise (float32 ray state with the
aberration polynomial evaluated in float32); pixels and histograms bit-exact
given the same float32 coordinates; field tolerances as for the other
beamlet-field tests; the reverse mode through the lens against central
differences of the oracle.  The batched path rejects the component."""
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


def test_adjoint_through_aberrated_lens(cuda):
    """Reverse mode through the aberrated lens (the state entering it is
    recomputed, its slope map has no closed-form inverse): per-ray input
    gradients and the lens focal length's gradient of a weighted sum of the
    outputs, against central differences of the oracle's polar-form series
    (<= 1e-4 normwise)."""
    import temgymcore_gb300 as t
    rng = np.random.default_rng(5)
    n = 4096
    x0, y0 = rng.uniform(-1e-3, 1e-3, n), rng.uniform(-1e-3, 1e-3, n)
    dx0, dy0 = rng.normal(0, 1e-3, n), rng.normal(0, 1e-3, n)
    v = [a.astype(np.float32).astype(np.float64) for a in (x0, y0, dx0, dy0)]
    coeffs = _coeffs(rng, 0.2, 3e-3)
    spec = [{"kind": "lens", "z": 0.2, "focal_length": 0.5},
            {"kind": "aberrated_lens", "z": 0.5, "focal_length": 0.2, "coeffs": coeffs},
            {"kind": "deflector", "z": 0.7, "def_x": 2e-4, "def_y": -1e-4},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (8, 8)}]
    wts = rng.normal(size=(5, n))
    wts[4] *= 1e-3  # the pathlength's weight
    f_t = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    xs = [torch.tensor(a, dtype=torch.float32, device=cuda, requires_grad=True) for a in v]
    model = [t.Lens(z=0.2, focal_length=0.5),
             t.AberratedLensKrivanek(z=0.5, focal_length=f_t, coeffs=t.KrivanekCoeffs(**coeffs)),
             t.Deflector(z=0.7, def_x=2e-4, def_y=-1e-4),
             t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(8, 8))]
    out = t.run_to_end(t.Ray(x=xs[0], y=xs[1], dx=xs[2], dy=xs[3], z=0.0, pathlength=0.0), model)
    W = [torch.tensor(w, device=cuda) for w in wts]
    loss = sum((W[i] * getattr(out, k).double()).sum() for i, k in enumerate(("x", "y", "dx", "dy")))
    loss = loss + (W[4] * out.pathlength).sum()
    loss.backward()

    def per_ray(vals, sp):
        o = oracle.run_to_end(ORay(*vals, 0.0, 0.0), sp)
        return (wts[0] * o.x + wts[1] * o.y + wts[2] * o.dx + wts[3] * o.dy
                + wts[4] * np.broadcast_to(o.pathlength, (n,)))
    for j, k in enumerate(("x", "y", "dx", "dy")):
        h = 1e-7 * (1e-3 if k in ("x", "y") else 1e-3)
        vp = [a.copy() for a in v]
        vm = [a.copy() for a in v]
        vp[j] += h
        vm[j] -= h
        fd = (per_ray(vp, spec) - per_ray(vm, spec)) / (2 * h)
        assert normwise_err(np_(xs[j].grad), fd) <= 1e-4, (k, normwise_err(np_(xs[j].grad), fd))

    def total(fv):
        sp = [dict(c) for c in spec]
        sp[1]["focal_length"] = fv
        return float(per_ray(v, sp).sum())
    fd_f = (total(0.2 + 1e-8) - total(0.2 - 1e-8)) / 2e-8
    assert abs(float(f_t.grad) - fd_f) <= 1e-4 * abs(fd_f), (float(f_t.grad), fd_f)


def test_batched_rejects_aberrated_lens(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace
    model = [t.AberratedLensKrivanek(z=0.5, focal_length=0.2, coeffs={"C30": 1e3}),
             t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(8, 8))]
    with pytest.raises(RuntimeError):
        BatchedTrace([model], [16])
    assert N.error_word() == 0
