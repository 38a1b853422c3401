"""GPU parity of the run.py utilities around run_to_end: the propagator call
and run_iter (tests/test_rays.py:15-39, tests/test_run.py:10-92 known
answers), the per-step Jacobians (run_iter with jacobian_transform equals
solve_model; custom_jacobian_matrix), run_with_grads (README.md:113-160
gradients and per-ray complex-step derivatives of the float64 oracle), and
inplace_sum (utils.py:83-114) against a serial loop.  Tolerances: float32 ray
state 1e-6 relative; derivatives 1e-4 normwise (float32 adjoint)."""
import numpy as np
import pytest
import torch

import oracle
from conftest import normwise_err
from oracle.rays import ORay

pytestmark = pytest.mark.gpu


def T():
    import temgymcore_gb300 as t
    return t


def _np(v):
    return v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)


def test_propagator_call_kats(kats, cuda):
    t = T()
    for c in kats["propagation"]["cases"]:
        x, y, dx, dy, z, pl = c["ray"]
        r = t.Ray(x=torch.tensor([x], device=cuda), y=torch.tensor([y], device=cuda),
                  dx=torch.tensor([dx], device=cuda), dy=torch.tensor([dy], device=cuda), z=z,
                  pathlength=torch.tensor([pl], dtype=torch.float64, device=cuda))
        for o in (t.FreeSpaceParaxial()(r, c["d"]), t.FreeSpaceParaxial.propagate(r, c["d"]),
                  t.FreeSpaceParaxial().with_distance(c["d"])(r)):
            got = [float(_np(o.x)[0]), float(_np(o.y)[0]), float(_np(o.dx)[0]), float(_np(o.dy)[0]),
                   float(o.z), float(_np(o.pathlength)[0])]
            np.testing.assert_allclose(got, c["expected"], rtol=1e-6, atol=1e-6)


def test_run_iter_kats(kats, cuda):
    t = T()
    from temgymcore_gb300.workloads import build_model
    ri = kats["run_iter"]
    x, y, dx, dy, z, pl = ri["ray"]
    r0 = t.Ray(x=x, y=y, dx=dx, dy=dy, z=z, pathlength=pl)
    model = build_model(ri["model"])
    steps = list(t.run_iter(r0, model))
    ref = list(oracle.run_iter(ORay(x, y, dx, dy, z, pl), ri["model"]))
    assert len(steps) == len(ref) == 2 * len(model)
    for (step, got), (_, want) in zip(steps, ref):
        for k in ("x", "y", "dx", "dy", "pathlength"):
            assert float(_np(getattr(got, k))) == pytest.approx(float(getattr(want, k)), rel=1e-6, abs=1e-6), k
        assert float(got.z) == pytest.approx(float(want.z), rel=1e-12)
    for i, comp in enumerate(model):  # the yielded propagator carries the distance
        assert float(steps[2 * i][0].distance) == pytest.approx(
            float(comp.z) - float((r0 if i == 0 else steps[2 * i - 1][1]).z), rel=1e-12)
    # no-propagation model: run_to_end equals composing the component calls
    x, y, dx, dy, z, pl = ri["noprop_ray"]
    r1 = t.Ray(x=x, y=y, dx=dx, dy=dy, z=z, pathlength=pl)
    m1 = build_model(ri["noprop_model"])
    out = t.run_to_end(r1, m1)
    ref = r1
    for c in m1:
        ref = c(ref)
    for k in ("x", "y", "dx", "dy", "pathlength"):
        assert float(_np(getattr(out, k))) == pytest.approx(float(_np(getattr(ref, k))), rel=1e-6)


def test_step_jacobians_equal_solve_model(cuda):
    t = T()
    from temgymcore_gb300.utils import custom_jacobian_matrix
    from temgymcore_gb300.workloads import build_model
    spec = [{"kind": "lens", "z": 0.1, "focal_length": 0.05},
            {"kind": "deflector", "z": 0.2, "def_x": 2e-4, "def_y": -1e-4},
            {"kind": "rotator", "z": 0.25, "angle": 23.0},
            {"kind": "biprism", "z": 0.3, "def_x": 5e-4},
            {"kind": "thicklens", "z_po": 0.4, "z_pi": 0.41, "focal_length": 0.2},
            {"kind": "detector", "z": 0.8, "pixel_size": (2e-5, 2e-5), "shape": (128, 128)}]
    model = build_model(spec)
    r = t.Ray(x=1e-4, y=-2e-4, dx=3e-3, dy=1e-3, z=0.0, pathlength=0.0)
    jacs = [custom_jacobian_matrix(j) for _, j in t.run_iter(r, model, transform=t.jacobian_transform)]
    np.testing.assert_allclose(np.stack(jacs), t.solve_model(r, model), rtol=1e-12, atol=1e-15)
    # their product is the model's ABCD, which calculate_derivatives also gives
    prod = np.eye(5)
    for j in jacs:
        prod = j @ prod
    np.testing.assert_allclose(prod, t.abcd_matrix(r, model), rtol=1e-12, atol=1e-15)
    (d1,) = t.calculate_derivatives(r, model, 1)
    np.testing.assert_allclose(custom_jacobian_matrix(d1), t.abcd_matrix(r, model), rtol=0, atol=0)
    with pytest.raises(NotImplementedError):
        t.calculate_derivatives(r, model, 2)


def test_run_with_grads_readme(kats, cuda):
    t = T()
    q = kats["readme_quickstart"]
    lens = t.Lens(z=0.5, focal_length=1.0)
    det = t.Detector(z=1.0, pixel_size=(0.01, 0.01), shape=(128, 128))
    ray = t.Ray(**q["ray"])
    value, grads = t.run_with_grads(ray, [lens, det], [lens.params.focal_length, lens.params.z,
                                                        ray.params.x])
    np.testing.assert_allclose([float(_np(grads[(lens, "focal_length")].x)), float(_np(grads[(lens, "z")].x))],
                               kats["readme_grads"]["dx_out_d_f_and_z"], rtol=1e-6)
    assert set(grads) == {(lens, "focal_length"), (lens, "z"), (ray, "x")}
    assert float(_np(grads[(ray, "x")].dx)) == pytest.approx(kats["readme_grads"]["ddx_out_dx_in"], abs=1e-6)
    assert float(_np(grads[(ray, "x")].dy)) == pytest.approx(kats["readme_grads"]["ddy_out_dx_in"], abs=1e-6)
    assert float(_np(value.x)) == pytest.approx(q["expected"]["x"], rel=1e-6)
    # d z_out / d(detector z) = 1; d pathlength_out / d pathlength_in = 1
    _, g2 = t.run_with_grads(ray, [lens, det], [det.params.z, ray.params.pathlength])
    assert float(_np(g2[(det, "z")].z)) == 1.0
    assert float(_np(g2[(ray, "pathlength")].pathlength)) == 1.0 and float(_np(g2[(ray, "pathlength")].x)) == 0.0
    with pytest.raises(RuntimeError):
        t.run_with_grads(ray, [lens, det], [t.Lens(z=0.1, focal_length=1.0).params.focal_length])


def test_run_with_grads_vector_rays_vs_complex_step(cuda):
    """Per-ray Jacobians of a chain with vector rays: parameter columns (N,)
    and the diagonal (N, N) blocks of the ray fields, against complex-step
    derivatives of the float64 oracle."""
    t = T()
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(3)
    n = 24
    w = {k: rng.normal(0, 1e-4, n).astype(np.float32) for k in ("x", "y", "dx", "dy")}
    spec = [{"kind": "lens", "z": 0.1, "focal_length": 0.05},
            {"kind": "deflector", "z": 0.2, "def_x": 2e-4, "def_y": -1e-4},
            {"kind": "detector", "z": 0.8, "pixel_size": (2e-5, 2e-5), "shape": (128, 128)}]
    model = build_model(spec)
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda), z=0.0,
                pathlength=0.0)
    value, grads = t.run_with_grads(ray, model, [model[0].params.focal_length, model[1].params.def_x,
                                                 ray.params.dx])
    h = 1e-30

    def cs(which, key):
        f = lambda a: np.asarray(a, np.float32).astype(np.complex128)  # noqa: E731
        d = {k: f(w[k]) for k in w}
        sp = [dict(c) for c in spec]
        if which == "ray":
            d[key] = d[key] + 1j * h
        else:
            sp[key[0]][key[1]] = sp[key[0]][key[1]] + 1j * h
        o = oracle.run_to_end(ORay(d["x"], d["y"], d["dx"], d["dy"], np.complex128(0), np.complex128(0)), sp)
        return {k: np.imag(getattr(o, k)) / h for k in ("x", "y", "dx", "dy", "pathlength")}

    for key, ref in (((model[0], "focal_length"), cs("param", (0, "focal_length"))),
                     ((model[1], "def_x"), cs("param", (1, "def_x")))):
        g = grads[key]
        for k in ("x", "y", "dx", "dy", "pathlength"):
            got = _np(getattr(g, k))
            assert got.shape == (n,)
            assert normwise_err(got, ref[k]) <= 1e-4 or np.max(np.abs(ref[k])) < 1e-12, (key[1], k)
    gk = [k for k in grads if k[-1] == "dx" and len(k) == 2 and not isinstance(k[0], t.Component)]
    assert len(gk) == 1
    ref = cs("ray", "dx")
    for k in ("x", "y", "dx", "dy", "pathlength"):
        blk = _np(getattr(grads[gk[0]], k))
        assert blk.shape == (n, n)
        assert np.count_nonzero(blk - np.diag(np.diag(blk))) == 0
        assert normwise_err(np.diag(blk), ref[k]) <= 1e-4 or np.max(np.abs(ref[k])) < 1e-12, k
    np.testing.assert_allclose(_np(value.x), _np(t.run_to_end(ray, model).x), rtol=0, atol=0)


def test_inplace_sum_matches_serial(cuda):
    from temgymcore_gb300.utils import inplace_sum
    rng = np.random.default_rng(6)
    n, h, w = 200_000, 37, 53
    py = rng.integers(-3, h + 3, n)
    px = rng.integers(-3, w + 3, n)
    mask = rng.random(n) < 0.8
    ref_i = np.zeros((h, w), np.int64)
    ref_f = np.zeros((h, w), np.float64)
    frame_i = rng.integers(-5, 6, n)
    frame_f = rng.normal(0, 1, n)
    for i in np.nonzero(mask & (py >= 0) & (py < h) & (px >= 0) & (px < w))[0]:
        ref_i[py[i], px[i]] += frame_i[i]
        ref_f[py[i], px[i]] += frame_f[i]
    buf = torch.zeros((h, w), dtype=torch.int64, device=cuda)
    inplace_sum(py, px, mask, frame_i, buf)
    np.testing.assert_array_equal(buf.cpu().numpy(), ref_i)
    bf = torch.zeros((h, w), dtype=torch.float64, device=cuda)
    inplace_sum(torch.tensor(py, device=cuda), torch.tensor(px, device=cuda), torch.tensor(mask, device=cuda),
                torch.tensor(frame_f, device=cuda), bf)
    np.testing.assert_allclose(bf.cpu().numpy(), ref_f, rtol=1e-12, atol=1e-12)
    host = np.ones((h, w), np.int32)   # a NumPy buffer is updated in place; no mask / frame = counts
    inplace_sum(py, px, None, None, host)
    cnt = np.ones((h, w), np.int32)
    ok = (py >= 0) & (py < h) & (px >= 0) & (px < w)
    np.add.at(cnt, (py[ok], px[ok]), 1)
    np.testing.assert_array_equal(host, cnt)
    inplace_sum(py[:0], px[:0], None, None, host)  # no hits: unchanged
    np.testing.assert_array_equal(host, cnt)
