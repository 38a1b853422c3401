"""GPU ray sources (source.py:82-188, utils.py:117-202) and decompose_Q_inv
(gaussian.py:35-89) against the oracle.  Deterministic sources match the
reference ray for ray (same count, ring radii and running angles; positions
within 4 ulp of the extent since CUDA's float64 sin/cos are within 2 ulp of
the host's); random sources are checked for count, support and uniformity;
decompose_Q_inv matches in waists and radii (1e-12 relative), reconstructs
Q^-1 and the reference test's input images, and gives theta modulo pi."""
import numpy as np
import pytest
import torch

from oracle import field as OF
from oracle import sources as OS

pytestmark = pytest.mark.gpu


def np_(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("num", [1, 2, 7, 100, 1000, 12345, 200001])
def test_deterministic_sources_match_reference(num, cuda):
    import temgymcore_gb300 as t
    ps = t.PointSource(z=0.1, semi_conv=3e-3, offset_xy=(1e-4, -2e-4))
    got = np_(ps.generate_array(num))
    ref = OS.point_source_array(num, 3e-3, (1e-4, -2e-4))
    assert got.shape == ref.shape
    np.testing.assert_array_equal(got[:, [0, 1, 4]], ref[:, [0, 1, 4]])
    np.testing.assert_allclose(got[:, 2:4], ref[:, 2:4], rtol=0, atol=4 * np.spacing(3e-3))
    pb = t.ParallelBeam(z=0.0, radius=2e-6, offset_xy=(5e-7, 0.0))
    got = np_(pb.generate_array(num))
    ref = OS.parallel_beam_array(num, 2e-6, (5e-7, 0.0))
    assert got.shape == ref.shape
    np.testing.assert_allclose(got[:, :2], ref[:, :2], rtol=0, atol=8 * np.spacing(2e-6))
    assert np.all(got[:, 2:4] == 0) and np.all(got[:, 4] == 1)
    yx = np_(t.concentric_rings(num, 0.5))
    np.testing.assert_allclose(yx, OS.concentric_rings(num, 0.5), rtol=0, atol=4 * np.spacing(0.5))


def test_make_rays_and_single_ray(cuda):
    import temgymcore_gb300 as t
    r = t.ParallelBeam(z=0.0, radius=0.0).make_rays(1)
    assert r.x.dim() == 0 and float(r.x) == 0.0 and float(r.dx) == 0.0
    r = t.PointSource(z=0.25, semi_conv=1e-3).make_rays(500)
    assert r.x.shape == (500,) or r.x.shape[0] > 400
    assert float(r.z) == 0.25
    out = t.run_to_end(r, [t.Lens(z=0.5, focal_length=0.2),
                           t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(64, 64))])
    assert torch.isfinite(out.x).all()


def test_random_sources(cuda):
    import temgymcore_gb300 as t
    n = 1_000_000
    a = np_(t.PointSource(z=0.0, semi_conv=2.0).generate_array(n, random=True, seed=7))
    assert a.shape == (n, 5)
    rr = np.hypot(a[:, 2], a[:, 3])
    assert rr.max() <= 2.0
    assert abs(np.mean(rr < 1.0) - 0.25) < 0.003  # uniform in area: P(r < R/2) = 1/4
    assert abs(a[:, 2].mean()) < 0.01 and abs(a[:, 3].mean()) < 0.01
    b = np_(t.PointSource(z=0.0, semi_conv=2.0).generate_array(n, random=True, seed=7))
    assert np.array_equal(a, b)
    c = np_(t.PointSource(z=0.0, semi_conv=2.0).generate_array(n, random=True, seed=8))
    assert not np.array_equal(a, c)
    yx = np_(t.random_coords(1000, seed=3))
    assert yx.shape == (1000, 2) and np.all(np.hypot(yx[:, 0], yx[:, 1]) < 1.0)


def _reconstruct(w1, w2, r1, r2, th, wl):
    return OF.Q_inv(np.stack([w1, w2], -1), np.stack([r1, r2], -1), np.full(np.size(w1), wl), th)


def test_decompose_q_inv(cuda):
    import temgymcore_gb300 as t
    wl = 1.3e-6
    params = [(1e-5, 3e-5, np.inf, np.inf, np.pi / 6), (1.2e-4, 5e-5, 0.0001, 0.1, -np.pi / 4),
              (1e-4, 3e-4, 0.01, np.inf, -np.pi / 3)]  # tests/test_gaussians.py:889-894
    rng = np.random.default_rng(0)
    for _ in range(200):
        params.append((rng.uniform(1e-5, 3e-4), rng.uniform(1e-5, 3e-4),
                       rng.choice([np.inf, rng.uniform(-1, 1)]), rng.choice([np.inf, rng.uniform(0.01, 2)]),
                       rng.uniform(-np.pi, np.pi)))
    p = np.array(params)
    q = OF.Q_inv(p[:, 0:2], p[:, 2:4], np.full(len(p), wl), p[:, 4])
    got = [np_(v) for v in t.decompose_Q_inv(q, wl)]
    ref = OF.decompose_Q_inv(q, wl)
    for g, r in zip(got[:4], ref[:4]):
        fin = np.isfinite(r)
        assert np.array_equal(np.isfinite(g), fin)
        np.testing.assert_allclose(g[fin], r[fin], rtol=1e-12)
    d = np.angle(np.exp(2j * (got[4] - ref[4]))) / 2  # theta modulo pi
    assert np.abs(d).max() < 1e-10
    # decompose_Q_inv returns R = 1 / Re(q) (gaussian.py:80-84) while
    # GaussianRay.q_inv uses -1 / R (gaussian.py:146-156): feeding the radii
    # back flips the real part (the reference's own round-trip test compares
    # amplitudes only), so the round trip is checked with -R
    q2 = _reconstruct(got[0], got[1], -got[2], -got[3], got[4], wl)
    np.testing.assert_allclose(q2, q, rtol=1e-10, atol=1e-12 * np.abs(q).max())
    # the reference test's image round trip (tests/test_gaussians.py:896-946)
    det = t.Detector(z=0.0, pixel_size=(1e-6, 1e-6), shape=(128, 128))
    for i in range(3):
        def ray(w, r, th):
            return t.GaussianRay(x=np.zeros(1), y=np.zeros(1), dx=np.zeros(1), dy=np.zeros(1), z=0.0,
                                 pathlength=np.zeros(1), amplitude=np.ones(1, np.complex64),
                                 waist_xy=np.array([w]), radii_of_curv=np.array([r]), wavelength=wl,
                                 theta=np.array([th]))
        a = np_(t.evaluate_gaussian_input_image(ray(p[i, 0:2], p[i, 2:4], p[i, 4]), det, method="fp64"))
        b = np_(t.evaluate_gaussian_input_image(ray([got[0][i], got[1][i]], [got[2][i], got[3][i]], got[4][i]),
                                                det, method="fp64"))
        np.testing.assert_allclose(np.abs(b), np.abs(a), rtol=1e-5, atol=1e-6)
