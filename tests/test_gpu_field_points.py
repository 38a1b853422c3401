"""GPU parity of the per-beam-ABCD field at arbitrary points:
propagate_misaligned_gaussian_jax_scan (gaussian.py:319-337, _beam_field
gaussian.py:276-316) and evaluate_misaligned_input_gaussian_jax_scan
(gaussian.py:410-427), complex128 out, against the float64 oracle's literal
restatement of the reference formula.  Tolerances: normwise relative error
<= 1e-12 and phase error <= 1e-11 rad at points brighter than 25% of the peak
(a NumPy restatement of the kernel's polynomial differs from the literal
formula by ~4e-15); against the complex64 grid API (exact pathlength phase
passed in): <= 1e-6 normwise."""
import numpy as np
import pytest
import torch

import oracle
from oracle import field as OF
from oracle.phase import phase_offset_exact

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _cmp(got, ref, tol=1e-12, ptol=1e-11):
    e = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert e <= tol, e
    bright = np.abs(ref) > 0.25 * np.max(np.abs(ref))
    ph = np.abs(np.angle(got[bright] * np.conj(ref[bright])))
    assert ph.max() <= ptol, ph.max()


def _inputs(astig, n=96, shape=(24, 40), seed=1):
    """Per-beam arguments of the beamlet workload (ABCD of each central ray from
    the oracle), the detector's pixel centres plus scattered points."""
    from temgymcore_gb300.workloads import beamlet_field
    w = beamlet_field(seed=seed, n_beams=n, det_shape=shape, det_px=4e-5, astigmatic=astig)
    r = w["rays"]
    x, y, dx, dy = (np.asarray(r[k], np.float64) for k in ("x", "y", "dx", "dy"))
    M = OF.beam_abcd(x, y, dx, dy, 0.0, w["model"])
    q1 = OF.Q_inv(np.asarray(r["waist_xy"]), np.asarray(r["radii_of_curv"]), r["wavelength"],
                  np.asarray(r["theta"]))
    k = np.full(n, 2 * np.pi / r["wavelength"])
    det = w["model"][-1]
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    X, Y = oracle.pixels_to_metres(det, yy.ravel(), xx.ravel())
    rng = np.random.default_rng(seed)
    extra = rng.uniform(-1, 1, (300, 2)) * np.abs(np.stack([X, Y], -1)).max()
    pts = np.concatenate([np.stack([X, Y], -1), extra])
    args = dict(amp=np.asarray(r["amplitude"], np.complex128), po=rng.uniform(-50, 50, n), q1=q1,
                A=M[:, 0:2, 0:2].copy(), B=M[:, 0:2, 2:4].copy(), C=M[:, 2:4, 0:2].copy(),
                D=M[:, 2:4, 2:4].copy(), e=M[:, 0:2, 4].copy(), f=M[:, 2:4, 4].copy(),
                r1m=np.stack([x, y], -1), t1m=np.stack([dx, dy], -1), k=k)
    return w, args, pts


def _ref(a, pts):
    q2 = OF.Qinv_ABCD(a["q1"], a["A"], a["B"], a["C"], a["D"])
    return OF.beam_field_pixels(a["amp"], a["po"], a["q1"], q2, a["r1m"], a["t1m"], a["A"], a["B"], a["e"],
                                a["f"], a["k"], pts).sum(axis=0)


def _call(a, pts, **over):
    from temgymcore_gb300.gaussian import propagate_misaligned_gaussian_jax_scan as prop
    v = dict(a, **over)
    return _np(prop(v["amp"], v["po"], v["q1"], v["A"], v["B"], v["C"], v["D"], v["e"], v["f"], v["r1m"],
                    v["t1m"], v["k"], pts))


@pytest.mark.parametrize("astig", [False, True])
def test_points_field_matches_oracle(astig, cuda):
    import temgymcore_gb300 as t
    _, a, pts = _inputs(astig)
    got = _call(a, pts)
    assert got.shape == (pts.shape[0],) and got.dtype == np.complex128
    _cmp(got, _ref(a, pts))
    # deterministic (chunk partials summed in a fixed order)
    np.testing.assert_array_equal(_call(a, pts), got)
    assert t._native.error_word() == 0


def test_points_field_equals_grid_api(cuda):
    """With the exactly reduced k*pathlength as phase_offset, the point API at
    the pixel centres is the complex64 grid API's float64 kernel."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays
    w, a, pts = _inputs(False)
    shape = w["model"][-1]["shape"]
    npx = shape[0] * shape[1]
    po = phase_offset_exact(a["k"], np.asarray(w["rays"]["pathlength"], np.float64))
    got = _call(a, pts[:npx], po=po)
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    ref = _np(plan.evaluate("fp64")).reshape(-1).astype(np.complex128)
    _cmp(got, ref, 1e-6, 1e-6)


def test_points_field_broadcast_edges_and_singular(cuda):
    from temgymcore_gb300.gaussian import propagate_misaligned_gaussian_jax_scan as prop
    _, a, pts = _inputs(False, n=40)
    # scalar k / phase_offset broadcast to every beam
    got = _call(a, pts, k=float(a["k"][0]), po=0.5)
    _cmp(got, _ref(dict(a, po=np.full(40, 0.5)), pts))
    # no beams: zeros; no points: empty
    z = _np(prop(a["amp"][:0], a["po"][:0], a["q1"][:0], a["A"][:0], a["B"][:0], a["C"][:0], a["D"][:0],
                 a["e"][:0], a["f"][:0], a["r1m"][:0], a["t1m"][:0], a["k"][:0], pts))
    assert z.shape == (pts.shape[0],) and not np.any(z)
    assert _call(a, pts[:0]).shape == (0,)
    # B = 0 (no propagation): B^-1 is zeroed, but (B (A Q1 + B))^-1 is not, so
    # the reference's field is NaN there; so is this one
    eye = np.broadcast_to(np.eye(2), (40, 2, 2)).copy()
    zero = np.zeros((40, 2, 2))
    sing = _call(a, pts[:50], A=eye, B=zero, C=zero, D=eye, e=np.zeros((40, 2)), f=np.zeros((40, 2)))
    ref = _ref(dict(a, A=eye, B=zero, C=zero, D=eye, e=np.zeros((40, 2)), f=np.zeros((40, 2))), pts[:50])
    assert np.all(np.isnan(ref)) and np.all(np.isnan(sing))


@pytest.mark.parametrize("astig", [False, True])
def test_input_points_field(astig, cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.gaussian import evaluate_misaligned_input_gaussian_jax_scan as ev
    from temgymcore_gb300.workloads import build_model, gaussian_rays, input_field
    w = input_field(seed=3, n_beams=200, grid_shape=(32, 48), px=2e-5, astigmatic=astig)
    r = w["rays"]
    n = 200
    q1 = OF.Q_inv(np.asarray(r["waist_xy"]), np.asarray(r["radii_of_curv"]), r["wavelength"],
                  np.asarray(r["theta"]))
    k = np.full(n, 2 * np.pi / r["wavelength"])
    po = phase_offset_exact(k, np.broadcast_to(np.asarray(r["pathlength"], np.float64), (n,)))
    r1m = np.stack([np.asarray(r["x"], np.float64), np.asarray(r["y"], np.float64)], -1)
    t1m = np.stack([np.broadcast_to(np.asarray(r["dx"], np.float64), (n,)),
                    np.broadcast_to(np.asarray(r["dy"], np.float64), (n,))], -1)
    amp = np.broadcast_to(np.asarray(r["amplitude"], np.complex128), (n,)).copy()
    from oracle.grid import grid_coords
    pts = grid_coords(w["grid"]).reshape(-1, 2)
    got = _np(ev(amp, po, q1, r1m, t1m, k, pts))
    ref = OF.input_beam_field_pixels(amp, q1, r1m, t1m, k, pts, po).sum(axis=0)
    _cmp(got, ref)
    grid = build_model([w["grid"]])[0]
    plan = t.FieldPlan(gaussian_rays(r), None, grid=grid)
    _cmp(got, _np(plan.evaluate("fp64")).reshape(-1).astype(np.complex128), 1e-6, 1e-6)
    assert t._native.error_word() == 0
