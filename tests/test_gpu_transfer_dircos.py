"""GPU: transfer-matrix kernels (transfer.py:6-112) against the oracle and the
reference's own cases (tests/test_transfer.py:7-130), and the fused chain
with the direction-cosine propagator (propagator.py:79-116) against the
oracle, forward and adjoint (complex step).  Transfer results are float64:
<= 1e-13 relative.  Direction-cosine rays: coordinates <= 1e-6 normwise
(float32 ray state), pathlength <= 1e-7 normwise (its per-ray part, large
at these slopes, is float32), gradients <= 1e-4."""
import math

import numpy as np
import pytest
import torch

import oracle
from oracle import transfer as OT
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu


def np_(t):
    return t.detach().cpu().numpy()


def _free(d):
    m = np.eye(5)
    m[0, 2] = m[1, 3] = d
    return m


def test_transfer_reference_cases(cuda):
    import temgymcore_gb300 as t
    # free space point source (tests/test_transfer.py:7-36)
    a = math.pi / 4
    c = np_(t.transfer_rays_pt_src((1.0, -2.0), (np.array([math.cos(a)]), np.array([math.sin(a)])), _free(5.0)))
    np.testing.assert_allclose(c[:, 0], [1 + 5 * math.cos(a), -2 + 5 * math.sin(a), math.cos(a), math.sin(a)],
                               atol=1e-12)
    # random integer matrix (tests/test_transfer.py:39-64)
    rng = np.random.RandomState(3)
    T = rng.randint(-5, 5, size=(5, 5)).astype(float)
    T[4, :] = [0, 0, 0, 0, 1]
    c = np_(t.transfer_rays_pt_src((0.7, -1.2), (np.array([0.3]), np.array([-0.4])), T))
    np.testing.assert_allclose(c[:, 0], T.dot([0.7, -1.2, 0.3, -0.4, 1.0])[:4], atol=1e-12)
    # identity batch, empty input, negative distance (tests/test_transfer.py:67-117)
    dxv, dyv = rng.randn(4), rng.randn(4)
    c = np_(t.transfer_rays_pt_src((0.5, -0.5), (dxv, dyv), np.eye(5)))
    assert c.shape == (4, 4)
    np.testing.assert_allclose(c[0], 0.5)
    np.testing.assert_allclose(c[2], dxv)
    assert tuple(t.transfer_rays_pt_src((1.0, 2.0), (np.zeros(0), np.zeros(0)), np.eye(5)).shape) == (4, 0)
    c = np_(t.transfer_rays_pt_src((1.0, 2.0), (np.array([0.1]), np.array([-0.2])), _free(-3.0)))
    np.testing.assert_allclose(c[:2, 0], [1.0 - 0.3, 2.0 + 0.6], atol=1e-12)
    # shape (tests/test_transfer.py:120-130)
    assert tuple(t.transfer_rays(np.zeros((10, 5)), np.zeros((7, 5, 5))).shape) == (10, 7, 5)
    with pytest.raises(IndexError):
        t.transfer_rays(np.zeros((3, 5)), np.zeros((0, 5, 5)))


def test_transfer_rays_matches_oracle(cuda):
    import temgymcore_gb300 as t
    rng = np.random.default_rng(5)
    rays = np.hstack([rng.normal(0, 1e-3, (3001, 4)), np.ones((3001, 1))])
    mats = rng.normal(0, 1, (11, 5, 5))
    got = np_(t.transfer_rays(rays, mats))
    ref = OT.transfer_rays(rays, mats)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13 * np.abs(ref).max())
    sx, sy = rng.normal(0, 1e-2, 5000), rng.normal(0, 1e-2, 5000)
    got = np_(t.transfer_rays_pt_src((1e-4, -2e-4), (sx, sy), mats[0]))
    np.testing.assert_allclose(got, OT.transfer_rays_pt_src((1e-4, -2e-4), (sx, sy), mats[0]),
                               rtol=1e-12, atol=1e-14)


def test_dircos_reference_case(cuda):
    """tests/test_rays.py:59-79 through FreeSpaceDirCosine()(ray, d)."""
    import temgymcore_gb300 as t
    x0, y0, dx0, dy0, z0, pl0 = 1.0, -1.0, 2.0, 3.0, 0.5, 10.0
    for d in (-7.3, 0.0, 4.1):
        new = t.FreeSpaceDirCosine()(t.Ray(x=x0, y=y0, dx=dx0, dy=dy0, z=z0, pathlength=pl0), d)
        n = math.sqrt(1.0 + dx0 ** 2 + dy0 ** 2)
        assert abs(float(new.x) - (x0 + (dx0 / n) / n * d)) < 1e-6
        assert abs(float(new.y) - (y0 + (dy0 / n) / n * d)) < 1e-6
        assert float(new.dx) == dx0 and float(new.dy) == dy0
        assert abs(float(new.z) - (z0 + d)) < 1e-12
        # pathlength: float64 base + float32 per-ray part d (N - 1)
        assert abs(float(new.pathlength) - (pl0 + d * n)) < 1e-6 * abs(d * n) + 1e-12


def _spec():
    return [{"kind": "lens", "z": 0.1, "focal_length": 0.4},
            {"kind": "deflector", "z": 0.2, "def_x": 1e-2, "def_y": -2e-2},
            {"kind": "biprism", "z": 0.3, "def_x": 5e-3},
            {"kind": "rotator", "z": 0.35, "angle": 20.0},
            {"kind": "detector", "z": 0.6, "pixel_size": (1e-3, 1e-3), "shape": (128, 128)}]


def test_dircos_chain_forward_and_adjoint(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(9)
    n = 8193
    w = {k: rng.normal(0, s, n).astype(np.float32) for k, s in (("x", 2e-3), ("y", 2e-3), ("dx", 0.2),
                                                                 ("dy", 0.2))}
    spec = _spec()
    xs = {k: torch.tensor(w[k], device=cuda, requires_grad=True) for k in w}
    out = t.run_to_end(t.Ray(x=xs["x"], y=xs["y"], dx=xs["dx"], dy=xs["dy"], z=0.0, pathlength=0.0),
                       build_model(spec), propagator=t.FreeSpaceDirCosine())
    ref = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], 0.0, 0.0), spec, "dircos")
    for k in ("x", "y", "dx", "dy"):
        assert normwise_err(np_(getattr(out, k)), getattr(ref, k)) <= 1e-6, k
    # the per-ray pathlength part is float32 and reaches ~0.33 m of the ~0.9 m
    # total at 0.2 rad slopes; a float32 emulation of the chain gives 3.5e-8
    assert normwise_err(np_(out.pathlength), ref.pathlength) <= 1e-7
    # differs from the paraxial chain at these slopes
    par = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], 0.0, 0.0), spec)
    assert normwise_err(ref.x, par.x) > 1e-2
    # adjoint of a random linear functional vs complex step on the oracle
    g = [rng.normal(0, 1, n) for _ in range(5)]
    loss = sum((torch.tensor(gi, device=cuda, dtype=torch.float64) * o.double()).sum()
               for gi, o in zip(g, (out.x, out.y, out.dx, out.dy, out.pathlength)))
    loss.backward()
    h = 1e-30
    for k in ("x", "y", "dx", "dy"):
        v = {q: np.asarray(w[q], np.float32).astype(np.complex128) for q in w}
        v[k] = v[k] + 1j * h
        o = oracle.run_to_end(ORay(v["x"], v["y"], v["dx"], v["dy"], np.complex128(0.0), np.complex128(0.0)),
                              spec, "dircos")
        d = [np.imag(getattr(o, f)) / h for f in ("x", "y", "dx", "dy", "pathlength")]
        refg = sum(gi * di for gi, di in zip(g, d))
        assert normwise_err(np_(xs[k].grad), refg) < 1e-4, k
    assert t._native.error_word() == 0


def test_dircos_rejected_by_batched_and_field(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.run import pack_model
    from temgymcore_gb300 import _native as N
    import ctypes as C
    from temgymcore_gb300.batched import TgBatchInfo
    model = [t.Lens(z=0.5, focal_length=0.2), t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(8, 8))]
    m, keep = pack_model(model, t.FreeSpaceDirCosine())
    arr = (N.TgModel * 1)(m)
    cnt = (C.c_int64 * 1)(16)
    info = TgBatchInfo()
    assert N.lib().tg_batch_plan(1, arr, cnt, None, 512, None, 0, C.byref(info)) == -2


def test_transfer_rays_double_float_range_and_fallback(cuda):
    """The double-float stack transfer against the float64 oracle at float64
    tolerance, for rays spanning many binades; rays with a component outside
    the double-float range ([2^-39, 2^62] or zero: tiny, huge) and matrices
    with such an entry take the float64 path and are just as close."""
    import temgymcore_gb300 as t
    rng = np.random.default_rng(6)
    n = 20000
    rays = np.hstack([rng.normal(0, 1, (n, 4)) * 10.0 ** rng.uniform(-9, 3, (n, 4)), np.ones((n, 1))])
    rays[:, :4][rng.random((n, 4)) < 0.05] = 0.0      # exact zeros
    rays[::97, 0] = 3e-15                             # below 2^-39: float64 path
    rays[::89, 2] = -7e20                             # above 2^62: float64 path
    rays[::61, 1] = 2.0 ** -39                        # the range's ends: double-float
    rays[::67, 3] = -(2.0 ** 62) / 1e6

    def in_range(v):
        a = np.abs(v)
        return (v == 0) | ((a >= 2.0 ** -39) & (a <= 2.0 ** 62))

    for scale in (1.0, 1e-14):                        # 1e-14: matrix entries outside the range
        mats = np.eye(5) + rng.normal(0, 0.5, (16, 5, 5))
        mats[:, 4, :] = [0, 0, 0, 0, 1]
        mats[-1, 0, 1] = scale                        # cumulative[0] is the last matrix itself
        cum = OT.accumulate_matrices_cumulative(mats)
        assert bool(np.all(in_range(cum))) == (scale == 1.0)   # which path the call takes
        got = np_(t.transfer_rays(rays, mats))
        ref = OT.transfer_rays(rays, mats)
        # per (ray, plane) record: error against the sum of the term magnitudes
        mag = np.einsum("pij,nj->npi", np.abs(cum), np.abs(rays))
        err = np.abs(got - ref)
        assert np.all(err <= 1e-13 * mag), (scale, float(np.max(err / np.maximum(mag, 1e-300))))
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13 * np.abs(ref).max())
