"""GPU parity of the Gaussian-beamlet field kernels against the float64
oracle (exact k*pathlength reduction).  Tolerances: field normwise relative
error <= 1e-4 (fast direct, split-BF16 tensor-core) and <= 5e-7 (float64
kernel, whose complex64 output alone rounds at ~6e-8); phase error <= 1e-4
rad (5e-7 rad for float64) at pixels brighter than 25% of the peak."""
import numpy as np
import pytest
import torch

from oracle import field as OF

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _cmp(got, ref, tol, ptol=1e-4):
    got = got.astype(np.complex128)
    e = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert e <= tol, e
    bright = np.abs(ref) > 0.25 * np.max(np.abs(ref))
    ph = np.abs(np.angle(got[bright] * np.conj(ref[bright])))
    assert ph.max() <= ptol, ph.max()
    return e, float(ph.max())


def _small(astig, n=256, shape=(64, 96), seed=0, det_px=4e-5):
    from temgymcore_gb300.workloads import beamlet_field
    return beamlet_field(seed=seed, n_beams=n, det_shape=shape, det_px=det_px, astigmatic=astig)


@pytest.mark.parametrize("astig", [False, True])
def test_field_methods_match_oracle(astig, cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    w = _small(astig)
    ref = OF.make_gaussian_image(w["rays"], w["model"])
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    assert plan.separable == (not astig)
    _cmp(_np(plan.evaluate("fp64")), ref, 5e-7, 5e-7)
    _cmp(_np(plan.evaluate("direct")), ref, 1e-4)
    if not astig:
        _cmp(_np(plan.evaluate("separable")), ref, 1e-4)
    assert t._native.error_word() == 0


def test_single_beams_phase_and_envelope(cuda):
    """One beam at a time: tilted, off-axis, astigmatic, curved, rotated grid."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    cases = [dict(x=1e-4, y=-2e-4, dx=1e-3, dy=-5e-4, wx=1e-4, wy=1e-4, R=np.inf, th=0.0),
             dict(x=0.0, y=0.0, dx=0.0, dy=0.0, wx=2e-4, wy=1e-4, R=np.inf, th=0.7),
             dict(x=-3e-4, y=1e-4, dx=2e-4, dy=1e-4, wx=1.5e-4, wy=1.5e-4, R=0.5, th=0.0)]
    for rot in (0.0, 30.0):
        spec = [{"kind": "lens", "z": 0.3, "focal_length": 0.4},
                {"kind": "deflector", "z": 0.4, "def_x": 1e-4, "def_y": 0.0},
                {"kind": "detector", "z": 1.0, "pixel_size": (2e-5, 2e-5), "shape": (48, 64),
                 "rotation": rot}]
        for c in cases:
            r = {"x": np.array([c["x"]]), "y": np.array([c["y"]]), "dx": np.array([c["dx"]]),
                 "dy": np.array([c["dy"]]), "z": 0.0, "pathlength": np.array([0.731]),
                 "amplitude": np.array([0.8 + 0.3j], np.complex64),
                 "waist_xy": np.array([[c["wx"], c["wy"]]]),
                 "radii_of_curv": np.array([[c["R"], c["R"]]]), "wavelength": 500e-9,
                 "theta": np.array([c["th"]])}
            ref = OF.make_gaussian_image(r, spec)
            plan = t.FieldPlan(gaussian_rays(r), build_model(spec), method="direct")
            _cmp(_np(plan.evaluate("direct")), ref, 1e-4)
            _cmp(_np(plan.evaluate("fp64")), ref, 5e-7, 5e-7)


def test_free_space_closed_form(kats, cuda):
    """tests/test_gaussians.py:229-273 closed form, sampled on a detector grid."""
    import temgymcore_gb300 as t
    g = kats["gauss_free_space"]
    w0, wl, L = g["w0"], g["wavelength"], g["L"]
    det = t.Detector(z=L, pixel_size=(1e-4, 1e-4), shape=(16, 16))
    ray = t.GaussianRay(x=np.zeros(1), y=np.zeros(1), dx=np.zeros(1), dy=np.zeros(1), z=0.0,
                        pathlength=np.zeros(1), amplitude=np.ones(1, np.complex64),
                        waist_xy=np.array([[w0, w0]]), radii_of_curv=np.array([[np.inf, np.inf]]),
                        wavelength=wl, theta=np.zeros(1))
    got = _np(t.make_gaussian_image(ray, [det], method="fp64"))
    k = 2 * np.pi / wl
    q = 1j * wl / (np.pi * w0 * w0)
    q2 = np.linalg.solve(np.eye(2) + L * np.eye(2) * q, q * np.eye(2))
    pref = 1.0 / np.sqrt(np.linalg.det(np.eye(2) + L * q * np.eye(2)))
    r2 = det.coords
    ref = (pref * np.exp(1j * (k / 2.0) * np.einsum("ni,ij,nj->n", r2, q2, r2))).reshape(16, 16)
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-7)
    got2 = _np(t.make_gaussian_image(ray, [det], method="separable"))
    np.testing.assert_allclose(got2, ref, rtol=1e-4, atol=1e-5)


def test_quadrant_of_tilted_beam(kats, cuda):
    import temgymcore_gb300 as t
    g = kats["gauss_quadrant"]
    det = t.Detector(z=g["z"], pixel_size=tuple(g["pixel_size"]), shape=tuple(g["shape"]))

    def img(dx, dy):
        ray = t.GaussianRay(x=np.zeros(1), y=np.zeros(1), dx=np.array([dx]), dy=np.array([dy]), z=0.0,
                            pathlength=np.zeros(1), amplitude=np.ones(1, np.complex64),
                            waist_xy=np.array([[g["w0"], g["w0"]]]),
                            radii_of_curv=np.array([[np.inf, np.inf]]), wavelength=g["wavelength"],
                            theta=np.zeros(1))
        return np.abs(_np(t.make_gaussian_image(ray, [det])))
    c = img(0.0, 0.0)
    cy, cx = np.unravel_index(np.argmax(c), c.shape)
    xc, yc = det.pixels_to_metres((cy, cx))
    tt = g["tilt"]
    for dx, dy in ((tt, tt), (tt, -tt), (-tt, tt), (-tt, -tt)):
        my, mx = np.unravel_index(np.argmax(img(dx, dy)), c.shape)
        xm, ym = det.pixels_to_metres((my, mx))
        assert np.sign(xm - xc) == np.sign(dx) and np.sign(ym - yc) == np.sign(dy)


@pytest.mark.parametrize("n,shape", [(1, (1, 1)), (3, (5, 37)), (130, (37, 53)), (300, (129, 7))])
def test_ragged_beams_and_detectors(n, shape, cuda):
    """Beam counts and detector shapes that are not multiples of any tile (the
    separable GEMM pads M, N and K; the direct kernels' last tiles are partial)."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    w = _small(False, n=n, shape=shape)
    ref = OF.make_gaussian_image(w["rays"], w["model"])
    assert ref.shape == shape and np.max(np.abs(ref)) > 0
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    assert plan.separable
    _cmp(_np(plan.evaluate("fp64")), ref, 5e-7, 5e-7)
    for meth in ("direct", "separable"):
        got = _np(plan.evaluate(meth))
        assert got.shape == shape
        _cmp(got, ref, 1e-4)
    assert t._native.error_word() == 0


def test_zero_beams_field_and_adjoint(cuda):
    """No beams: every method returns a zero image; the adjoint returns empty
    per-beam gradients and zero per-step sums (the reference's chunked sum
    over an empty beam set is the zero image)."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    w = _small(False, n=8, shape=(9, 11))
    rays0 = {k: (v[:0] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == 8 else v)
             for k, v in w["rays"].items()}
    plan = t.FieldPlan(gaussian_rays(rays0), build_model(w["model"]))
    for meth in ("direct", "separable", "fp64"):
        img = _np(plan.evaluate(meth))
        assert img.shape == (9, 11) and not np.any(img), meth
    for meth in ("direct", "separable"):
        g = plan.vjp(torch.ones(plan.shape, dtype=torch.complex64, device=cuda), method=meth)
        for k in ("amplitude", "pathlength", "x", "y", "dx", "dy"):
            assert g[k].numel() == 0, (meth, k)
        assert not torch.any(g["raw"]), meth
    assert t._native.error_word() == 0


def test_separable_rejects_astigmatic_beams(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    w = _small(True, n=64, shape=(32, 32))
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    assert not plan.separable and plan.method == "direct"
    t._native.error_word()
    plan.evaluate("separable")
    assert t._native.error_word() & 0x10


def test_full_config_properties(cuda):
    """Full size (16,384 beams, 512 x 512): separable GEMM vs the fp64 kernel on all pixels,
    direct vs oracle on a pixel sample, astigmatic direct vs oracle sample."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    w = beamlet_field(seed=0)
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    assert plan.separable
    f64 = _np(plan.evaluate("fp64").clone()).astype(np.complex128)
    sep = _np(plan.evaluate("separable").clone())
    e = np.max(np.abs(sep - f64)) / np.max(np.abs(f64))
    assert e < 1e-4, e
    rng = np.random.default_rng(0)
    idx = rng.choice(512 * 512, 64, replace=False)
    ref = OF.make_gaussian_image(w["rays"], w["model"], pixel_index=idx, chunk=2048)
    e2 = np.max(np.abs(f64.reshape(-1)[idx] - ref)) / np.max(np.abs(ref))
    assert e2 < 1e-7, e2
    dire = _np(plan.evaluate("direct").clone()).reshape(-1)[idx]
    assert np.max(np.abs(dire - ref)) / np.max(np.abs(ref)) < 1e-4


def test_one_call_field_entry_points(cuda):
    """tg_field_direct / tg_field_separable (prep + eval in one call) equal the
    two-call FieldPlan results."""
    import ctypes as C
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.gaussian import BeamSet, TgBeams, TgPixelMap, pixel_map
    from temgymcore_gb300.run import pack_model
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    for name in ("tg_field_direct", "tg_field_separable"):
        N.register(name, C.c_int, [C.POINTER(N.TgModel), C.POINTER(TgBeams), C.POINTER(TgPixelMap), C.c_void_p,
                                   C.c_void_p, C.c_size_t, C.c_void_p])
    w = _small(False)
    model = build_model(w["model"])
    plan = t.FieldPlan(gaussian_rays(w["rays"]), model)
    beams = BeamSet(gaussian_rays(w["rays"]), cuda)
    pm = pixel_map(model[-1])
    m, keep = pack_model(model)
    for name, meth in (("tg_field_direct", "direct"), ("tg_field_separable", "separable")):
        out = torch.empty(plan.shape, dtype=torch.complex64, device=cuda)
        N.check(getattr(N.lib(), name)(C.byref(m), C.byref(beams.struct()), C.byref(pm),
                                       torch.view_as_real(out).data_ptr(), plan.ws_ptr, plan.ws_bytes,
                                       N.stream_ptr()))
        ref = plan.evaluate(meth).clone()
        torch.cuda.synchronize()
        assert torch.equal(out, ref), name
