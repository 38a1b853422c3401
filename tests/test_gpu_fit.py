"""Device-resident 4D-STEM fit: forward parity, gradient parity (complex-step
and central finite differences on the float64 oracle), CUDA-graph replay,
convergence.  Tolerances: detector positions <= 1e-6 normwise; gradients
within 1e-4 of the summed per-ray magnitudes plus 1e-3 relative."""
import numpy as np
import pytest
import torch

import oracle
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu


def _setup(cuda, scan=(6, 5), rays=512, seed=0):
    import temgymcore_gb300 as t
    from temgymcore_gb300.fit import StemFit
    from temgymcore_gb300.workloads import stem_fit
    w = stem_fit(seed=seed, scan=scan, rays_per_probe=rays)
    ray = t.Ray(x=w["x"], y=w["y"], dx=w["dx"], dy=w["dy"], z=0.0, pathlength=0.0)
    fit = StemFit(ray, w["rows"], w["cols"], w["gap"], w["theta0"])
    fit.set_targets(w["theta_true"])
    return w, fit


def _oracle_det(w, theta, h=None, hidx=None):
    """Detector x, y (n_probes, n) from the oracle, optional complex step."""
    from temgymcore_gb300.workloads import stem_fit_probe_spec
    th = np.asarray(theta, dtype=np.complex128 if h else np.float64).copy()
    if h:
        th[hidx] += 1j * h
    sg, spec = stem_fit_probe_spec(w, th, 0)
    rows, cols = w["rows"], w["cols"]
    yy, xx = np.meshgrid(np.arange(rows), np.arange(cols), indexing="ij")
    spx, spy = oracle.pixels_to_metres(sg, yy.ravel(), xx.ravel())
    dt = np.complex128 if h else np.float64
    r0 = ORay(w["x"].astype(dt), w["y"].astype(dt), w["dx"].astype(dt), w["dy"].astype(dt),
              np.asarray(0.0, dt), np.asarray(0.0, dt))
    X, Y = [], []
    for p in range(rows * cols):
        sp = [dict(c) for c in spec]
        for c in sp:
            if c["kind"] in ("scanner", "descanner"):
                c["scan_pos_x"], c["scan_pos_y"] = spx[p], spy[p]
        o = oracle.run_to_end(r0, sp)
        X.append(o.x)
        Y.append(o.y)
    return np.array(X), np.array(Y)


def test_forward_matches_oracle(cuda):
    w, fit = _setup(cuda)
    gx, gy = fit.forward(w["theta_true"])
    ox, oy = _oracle_det(w, w["theta_true"])
    assert normwise_err(gx.cpu().numpy(), ox) <= 1e-6
    assert normwise_err(gy.cpu().numpy(), oy) <= 1e-6


def test_gradient_matches_complex_step_and_fd(cuda):
    w, fit = _setup(cuda)
    out = fit.loss_grad().cpu().numpy()
    tx = fit.tx.cpu().numpy().astype(np.float64)
    ty = fit.ty.cpu().numpy().astype(np.float64)
    ox, oy = _oracle_det(w, w["theta0"])
    loss_ref = np.sum((ox - tx) ** 2 + (oy - ty) ** 2)
    assert abs(out[0] - loss_ref) <= 1e-4 * loss_ref
    h = 1e-30
    th0 = w["theta0"]
    for j in range(21):
        cx, cy = _oracle_det(w, th0, h, j)
        dxj, dyj = np.imag(cx) / h, np.imag(cy) / h
        contrib = 2 * (np.real(cx) - tx) * dxj + 2 * (np.real(cy) - ty) * dyj
        ref = contrib.sum()
        mag = np.abs(contrib).sum()
        assert abs(out[1 + j] - ref) <= 1e-4 * mag + 1e-3 * abs(ref), (j, out[1 + j], ref, mag)
        if j in (0, 1, 2, 5, 10):  # central finite differences, h = 1e-4 relative
            hh = 1e-4 * abs(th0[j])
            tp, tm = th0.copy(), th0.copy()
            tp[j] += hh
            tm[j] -= hh
            lp = sum(np.sum((a - b) ** 2) for a, b in zip(_oracle_det(w, tp), (tx, ty)))
            lm = sum(np.sum((a - b) ** 2) for a, b in zip(_oracle_det(w, tm), (tx, ty)))
            fd = (lp - lm) / (2 * hh)
            assert abs(fd - ref) <= 1e-5 * mag + 1e-4 * abs(ref), (j, fd, ref)


def test_graph_replay_equals_eager_and_converges(cuda):
    from temgymcore_gb300.workloads import stem_fit
    w, fa = _setup(cuda, scan=(32, 32), rays=1024)
    _, fb = _setup(cuda, scan=(32, 32), rays=1024)
    sc = np.abs(w["theta0"])
    sc[sc < 1e-2] = 1e-3  # off-diagonal descan entries: absolute scale
    for f in (fa, fb):
        f.scale.copy_(torch.as_tensor(sc))
    fa.fit(5, lr=1e-3, use_graph=True)
    fb.fit(5, lr=1e-3, use_graph=False)
    torch.cuda.synchronize()
    assert torch.equal(fa.theta, fb.theta)
    hist = fa.fit(195, lr=1e-3, use_graph=True).cpu().numpy()
    out = fa.loss_grad().cpu().numpy()
    assert out[0] < 1e-4 * hist[0], (hist[0], out[0])
    assert np.all(np.isfinite(fa.theta.cpu().numpy()))
    # the detector positions determine six combinations of the 21 parameters
    # (tests/test_fit_identifiability.py); those are recovered
    got, ref = fa.identifiable(), fa.identifiable(w["theta_true"])
    assert np.max(np.abs(got - ref) / np.abs(ref)) <= 1e-3, (got, ref)


def test_fused_step_equals_loss_grad_then_adam(cuda):
    """tg_stem_fit_step (two launches, Adam in the reduction's last block)
    gives bit-identical parameters, moments and outputs to tg_stem_fit_loss_grad
    followed by tg_adam_step."""
    w, fa = _setup(cuda, scan=(16, 16), rays=512)
    _, fb = _setup(cuda, scan=(16, 16), rays=512)
    sc = np.abs(w["theta0"])
    sc[sc < 1e-2] = 1e-3
    for f in (fa, fb):
        f.scale.copy_(torch.as_tensor(sc))
    for _ in range(5):
        fa.step(lr=2e-3)
        fb.loss_grad()
        fb.adam(lr=2e-3)
    torch.cuda.synchronize()
    assert torch.equal(fa.theta, fb.theta)
    assert torch.equal(fa.m, fb.m) and torch.equal(fa.v, fb.v) and torch.equal(fa.t, fb.t)
    assert torch.equal(fa.out, fb.out)
