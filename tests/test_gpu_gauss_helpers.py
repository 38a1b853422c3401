"""GPU parity of the Gaussian-beam helpers: GaussianRay.q_inv / Q_inv
(gaussian.py:138-177), Qinv_ABCD (gaussian.py:92-96), zR / w_z / R /
q_inv(z, w0, wl) / gaussian_beam (gaussian.py:13-32, 99-109), against the
float64 oracle, LAPACK's solve and the reference's own known answers
(tests/test_gaussians.py:167-226).  Tolerances: 1e-15 relative for the
rational helpers (one or two roundings apart: products and sums may fuse),
1e-14 for the 2x2 solves, 1e-13 for the complex exponential."""
import numpy as np
import pytest
import torch

from oracle import field as OF

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _normwise(got, ref):
    """Per 2x2 system: max |got - ref| / max |ref|."""
    n = int(np.prod(ref.shape[:-2]))
    d = np.abs(got - ref).reshape(n, -1).max(axis=1)
    return d / np.abs(ref).reshape(n, -1).max(axis=1)


def _beams(n, seed=0):
    import temgymcore_gb300 as t
    rng = np.random.default_rng(seed)
    waist = rng.uniform(1e-9, 1e-6, (n, 2))
    radii = rng.uniform(0.01, 10.0, (n, 2)) * rng.choice([-1, 1], (n, 2))
    radii[rng.random((n, 2)) < 0.3] = np.inf
    wl = rng.uniform(1e-12, 1e-9, n)
    theta = rng.uniform(0, np.pi, n)
    r = t.GaussianRay(x=np.zeros(n), y=np.zeros(n), dx=np.zeros(n), dy=np.zeros(n), z=0.0,
                      pathlength=np.zeros(n), amplitude=np.ones(n, np.complex64), waist_xy=waist,
                      radii_of_curv=radii, wavelength=wl, theta=theta)
    return r, waist, radii, wl, theta


def test_beam_q_inv_and_Q_inv(cuda):
    import temgymcore_gb300 as t
    n = 1000
    r, waist, radii, wl, theta = _beams(n)
    qx, qy = r.q_inv
    rx, ry = OF.q_inv(waist, radii, wl)
    assert qx.shape == (n,) and qx.dtype == torch.complex128
    np.testing.assert_allclose(_np(qx), rx, rtol=1e-15, atol=0)
    np.testing.assert_allclose(_np(qy), ry, rtol=1e-15, atol=0)
    Q = r.Q_inv
    ref = OF.Q_inv(waist, radii, wl, theta)
    assert Q.shape == (n, 2, 2)
    scale = np.abs(ref).reshape(n, -1).max(axis=1)[:, None, None]
    assert np.max(np.abs(_np(Q) - ref) / scale) <= 1e-15
    # Q^-1 is symmetric, and decompose_Q_inv takes it back to the beam
    np.testing.assert_array_equal(_np(Q[:, 0, 1]), _np(Q[:, 1, 0]))
    wx, wy, _, _, _ = t.decompose_Q_inv(Q, torch.tensor(wl))
    big, small = np.maximum(waist[:, 0], waist[:, 1]), np.minimum(waist[:, 0], waist[:, 1])
    np.testing.assert_allclose(_np(wx), big, rtol=1e-9)
    np.testing.assert_allclose(_np(wy), small, rtol=1e-9)
    # one beam given as (2,) vectors: scalars, as waist_xy.T unpacks
    one = t.GaussianRay(x=0.0, y=0.0, dx=0.0, dy=0.0, z=0.0, pathlength=0.0, amplitude=1.0,
                        waist_xy=np.array([1e-6, 2e-6]), radii_of_curv=np.array([np.inf, 1.0]),
                        wavelength=5e-7, theta=0.0)
    a, b = one.q_inv
    assert a.shape == () and b.shape == ()
    assert complex(a) == pytest.approx(1j * 5e-7 / (np.pi * 1e-12), rel=1e-15)
    assert complex(b) == pytest.approx(-1.0 + 1j * 5e-7 / (np.pi * 4e-12), rel=1e-15)
    assert t._native.error_word() == 0


def test_qinv_abcd_identity_and_solve(cuda):
    from temgymcore_gb300.gaussian import Qinv_ABCD
    eye, z = np.eye(2), np.zeros((2, 2))
    q1 = np.array([[2j, 0], [0, 3j]])
    # identity ABCD returns Q1 (tests/test_gaussians.py:218-226)
    np.testing.assert_allclose(_np(Qinv_ABCD(q1, eye, z, z, eye)), q1, rtol=1e-12, atol=0)
    rng = np.random.default_rng(4)
    n = 4096
    A, B, C, D = (rng.normal(0, 1, (n, 2, 2)) for _ in range(4))
    A[:64] = [[0.0, 1.0], [1.0, 0.0]]        # forces the row swap of the partial pivot
    B[:64] *= 1e-3
    Q = rng.normal(0, 1, (n, 2, 2)) + 1j * rng.normal(0, 1, (n, 2, 2))
    got = _np(Qinv_ABCD(Q, A, B, C, D))
    ref = np.linalg.solve(A + B @ Q, C + D @ Q)      # LAPACK gesv, as jnp.linalg.solve on the CPU
    cond = np.maximum(np.linalg.cond(A + B @ Q), 1.0)
    err = _normwise(got, ref)
    assert np.all(err <= 1e-14 * cond), float(np.max(err / cond))
    assert np.all(_normwise(got, OF.Qinv_ABCD(Q, A, B, C, D)) <= 1e-14 * cond)
    # broadcast: one ABCD for every Q, and a (3, 5) batch of Q
    Qb = Q[:15].reshape(3, 5, 2, 2)
    gb = _np(Qinv_ABCD(Qb, A[0], B[0], C[0], D[0]))
    assert gb.shape == (3, 5, 2, 2)
    rb = np.linalg.solve(A[0] + B[0] @ Qb, C[0] + D[0] @ Qb)
    assert np.all(_normwise(gb, rb) <= 1e-14 * np.maximum(np.linalg.cond(A[0] + B[0] @ Qb), 1.0).reshape(-1))
    with pytest.raises(NotImplementedError):
        Qinv_ABCD(Q[:2], A[:2] + 1j, B[:2], C[:2], D[:2])


def test_free_space_q_transform(cuda):
    """Free space over L: Q2 = Q1 (I + L Q1)^-1, i.e. 1/q2 = 1/(q1 + L) per axis."""
    from temgymcore_gb300.gaussian import Qinv_ABCD, q_inv
    w0, wl, L = 1e-4, 5e-7, 0.3
    q1 = complex(_np(q_inv(0.0, w0, wl)))
    Q1 = np.diag([q1, q1])
    got = _np(Qinv_ABCD(Q1, np.eye(2), L * np.eye(2), np.zeros((2, 2)), np.eye(2)))
    want = 1.0 / (1.0 / q1 + L)
    np.testing.assert_allclose(np.diag(got), [want, want], rtol=1e-13)
    # and that is the beam at distance L from its waist
    # (q_inv(z, w0, wl) writes the curvature term as -1/R, the ABCD law gives +1/R)
    np.testing.assert_allclose(-np.conj(want), _np(q_inv(L, w0, wl)), rtol=1e-9)


def test_profile_helpers_kats_and_oracle(cuda):
    from temgymcore_gb300.gaussian import R, gaussian_beam, q_inv, w_z, zR
    w0, wl = 1e-3, 500e-9  # tests/test_gaussians.py:167-203
    zr = float(_np(zR(w0, wl)))
    assert zr == pytest.approx(np.pi * w0 * w0 / wl, rel=1e-9)
    assert float(_np(w_z(w0, 0.0, zr))) == pytest.approx(w0, rel=1e-9)
    assert float(_np(w_z(w0, zr, zr))) == pytest.approx(w0 * np.sqrt(2.0), rel=1e-9)
    assert float(_np(R(zr, zr))) == pytest.approx(2 * zr, rel=1e-9)
    assert np.isinf(float(_np(R(0.0, zr))))
    assert complex(_np(q_inv(0.0, w0, wl))) == pytest.approx(1j * wl / (np.pi * w0 * w0), rel=1e-12)
    want = -(1.0 / (2 * zr)) + 1j * wl / (np.pi * (w0 * np.sqrt(2.0)) ** 2)
    assert complex(_np(q_inv(zr, w0, wl))) == pytest.approx(want, rel=1e-12)
    k = 2 * np.pi / wl  # tests/test_gaussians.py:206-214
    assert complex(_np(gaussian_beam(0.0, 0.0, 1j * 1e-6, k))) == pytest.approx(1.0, rel=1e-12)
    assert complex(_np(gaussian_beam(1e-3, -2e-3, 1j * 1e-6, k, offset_x=-1e-3, offset_y=2e-3))) == \
        pytest.approx(1.0, rel=1e-12)
    # elementwise over arrays (broadcast) against the oracle
    rng = np.random.default_rng(5)
    z = rng.uniform(-2, 2, 5000)
    z[:50] = rng.uniform(-1e-11, 1e-11, 50)   # the focus branch
    w0s = rng.uniform(1e-9, 1e-3, 5000)
    wls = rng.uniform(1e-12, 1e-6, 5000)
    zrs = OF.zR(w0s, wls)
    np.testing.assert_allclose(_np(zR(w0s, wls)), zrs, rtol=1e-15, atol=0)
    np.testing.assert_allclose(_np(w_z(w0s, z, zrs)), OF.w_z(w0s, z, zrs), rtol=1e-15, atol=0)
    rr = _np(R(z, zrs))
    np.testing.assert_array_equal(np.isinf(rr), np.isinf(OF.R_of_z(z, zrs)))
    fin = np.isfinite(rr)
    np.testing.assert_allclose(rr[fin], OF.R_of_z(z, zrs)[fin], rtol=1e-15, atol=0)
    np.testing.assert_allclose(_np(q_inv(z, w0s, wls)), OF.q_inv_z(z, w0s, wls), rtol=2e-15, atol=0)
    x, y = rng.normal(0, 1e-4, (2, 5000))
    qs = OF.q_inv_z(z, 1e-4, 5e-7)
    kk = 2 * np.pi / 5e-7
    got = _np(gaussian_beam(x, y, qs, kk, offset_x=1e-5, offset_y=-2e-5))
    ref = OF.gaussian_beam(x, y, qs, kk, offset_x=1e-5, offset_y=-2e-5)
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    assert zR(w0s[:0], wls[:0]).shape == (0,)
