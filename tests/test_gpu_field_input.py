"""GPU parity of the input-plane beamlet field (evaluate_gaussian_input_image,
gaussian.py:372-427) against the float64 oracle, plus the reference's own
input-image checks (tests/test_gaussians.py:736-786, 818-877) run through the
GPU API.  Tolerances as for the detector field: normwise relative error
<= 1e-4 for the fast direct and split-BF16 tensor-core sums, <= 5e-7 for the
float64 kernel; phase error <= 1e-4 rad (5e-7 rad for float64) at pixels
brighter than 25% of the peak."""
import numpy as np
import pytest

from oracle import field as OF
from oracle.grid import grid_coords

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


@pytest.mark.parametrize("astig", [False, True])
def test_input_field_matches_oracle(astig, cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays, input_field
    w = input_field(seed=3, n_beams=512, grid_shape=(64, 96), px=2e-5, astigmatic=astig)
    ref = OF.evaluate_gaussian_input_image(w["rays"], w["grid"])
    grid = build_model([w["grid"]])[0]
    plan = t.FieldPlan(gaussian_rays(w["rays"]), None, grid=grid)
    assert plan.separable == (not astig)
    _cmp(_np(plan.evaluate("fp64")), ref, 5e-7, 5e-7)
    _cmp(_np(plan.evaluate("direct")), ref, 1e-4)
    if not astig:
        _cmp(_np(plan.evaluate("separable")), ref, 1e-4)
    img = t.evaluate_gaussian_input_image(gaussian_rays(w["rays"]), grid)
    _cmp(_np(img), ref, 1e-4)
    assert t._native.error_word() == 0


def _one_beam(t, x0, y0, dx, dy, wavelength=500e-9, waist=(1e-4, 1e-4), theta=0.0, pl=0.0):
    return t.GaussianRay(x=np.array([x0]), y=np.array([y0]), dx=np.array([dx]), dy=np.array([dy]),
                         z=0.0, pathlength=np.array([pl]), amplitude=np.array([1.0 + 0j]),
                         waist_xy=np.array([list(waist)]), radii_of_curv=np.array([[np.inf, np.inf]]),
                         wavelength=wavelength, theta=np.array([theta]))


def test_input_field_phase_ramp(cuda):
    """tests/test_gaussians.py:736-786 through the GPU API: zero phase at the
    beam centre and a phase slope k * tilt along rows and columns."""
    import temgymcore_gb300 as t
    det = t.Detector(z=0.0, pixel_size=(1e-5, 1e-5), shape=(512, 512))
    xy = grid_coords({"kind": "detector", "z": 0.0, "pixel_size": (1e-5, 1e-5),
                      "shape": (512, 512)}).reshape(512, 512, 2)
    det_x, det_y = xy[0, :, 0], xy[:, 0, 1]
    ix = iy = 256
    wl = 500e-9
    k = 2 * np.pi / wl
    for dx, dy in ((2e-4, 0.0), (0.0, -1e-4), (1.5e-4, -1.0e-4)):
        ray = _one_beam(t, det_x[ix], det_y[iy], dx, dy, wl)
        for method in ("direct", "separable"):
            img = _np(t.evaluate_gaussian_input_image(ray, det, method=method)).astype(np.complex128)
            assert abs(np.angle(img[iy, ix])) < 1e-5, method
            rp = np.unwrap(np.angle(img[iy, :]))
            cp = np.unwrap(np.angle(img[:, ix]))
            sx = (rp[ix + 8] - rp[ix - 8]) / (det_x[ix + 8] - det_x[ix - 8])
            sy = (cp[iy + 8] - cp[iy - 8]) / (det_y[iy + 8] - det_y[iy - 8])
            np.testing.assert_allclose(sx, k * dx, rtol=2e-2, atol=1e-3)
            np.testing.assert_allclose(sy, k * dy, rtol=2e-2, atol=1e-3)


def test_input_field_astigmatic_rotation(cuda):
    """tests/test_gaussians.py:818-877 through the GPU API: the major axis of
    the intensity follows theta (direct sum: the rotated beam is not
    separable)."""
    import temgymcore_gb300 as t
    det = t.Detector(z=0.0, pixel_size=(1e-5, 1e-5), shape=(512, 512))
    xy = grid_coords({"kind": "detector", "z": 0.0, "pixel_size": (1e-5, 1e-5),
                      "shape": (512, 512)}).reshape(512, 512, 2)
    X, Y = xy[..., 0], xy[..., 1]
    for th in (np.pi / 3, np.pi / 6, 0.0, -np.pi / 6, -np.pi / 3, -np.pi / 2 + 0.1):
        img = _np(t.evaluate_gaussian_input_image(_one_beam(t, 0.0, 0.0, 0.0, 0.0, theta=th,
                                                            waist=(2e-4, 1e-4)), det))
        inten = np.abs(img.astype(np.complex128)) ** 2
        wsum = inten.sum() + 1e-30
        xb, yb = (inten * X).sum() / wsum, (inten * Y).sum() / wsum
        cxx = (inten * (X - xb) ** 2).sum() / wsum
        cyy = (inten * (Y - yb) ** 2).sum() / wsum
        cxy = (inten * (X - xb) * (Y - yb)).sum() / wsum
        vals, vecs = np.linalg.eigh(np.array([[cxx, cxy], [cxy, cyy]]))
        v = vecs[:, np.argmax(vals)]
        phi = (np.arctan2(v[1], v[0]) + np.pi / 2) % np.pi - np.pi / 2
        assert abs(np.arctan2(np.sin(phi - th), np.cos(phi - th))) < 0.1, th


def test_input_field_single_beams_vs_oracle(cuda):
    """Tilted, off-axis, astigmatic and curved single beams with a large
    pathlength phase, on a rotated grid."""
    import temgymcore_gb300 as t
    for rot in (0.0, 25.0):
        gd = {"kind": "detector", "z": 0.0, "pixel_size": (2e-5, 2e-5), "shape": (48, 64),
              "rotation": rot}
        from temgymcore_gb300.workloads import build_model
        grid = build_model([gd])[0]
        for c in (dict(x=1e-4, y=-2e-4, dx=1e-3, dy=-5e-4, w=(1e-4, 1e-4), R=np.inf, th=0.0),
                  dict(x=0.0, y=0.0, dx=0.0, dy=0.0, w=(2e-4, 1e-4), R=np.inf, th=0.7),
                  dict(x=-3e-4, y=1e-4, dx=2e-4, dy=1e-4, w=(1.5e-4, 1.5e-4), R=0.5, th=0.0)):
            r = {"x": np.array([c["x"]]), "y": np.array([c["y"]]), "dx": np.array([c["dx"]]),
                 "dy": np.array([c["dy"]]), "z": 0.0, "pathlength": np.array([0.731]),
                 "amplitude": np.array([0.8 + 0.3j], np.complex64), "waist_xy": np.array([c["w"]]),
                 "radii_of_curv": np.array([[c["R"], c["R"]]]), "wavelength": 500e-9,
                 "theta": np.array([c["th"]])}
            ref = OF.evaluate_gaussian_input_image(r, gd)
            from temgymcore_gb300.workloads import gaussian_rays
            plan = t.FieldPlan(gaussian_rays(r), None, "direct", grid=grid)
            _cmp(_np(plan.evaluate("direct")), ref, 1e-4)
            _cmp(_np(plan.evaluate("fp64")), ref, 5e-7, 5e-7)
