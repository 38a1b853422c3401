"""Krivanek aberrations (aberrations.py:42-108, components.py:177-215) on the
CPU: the oracle's literal polar-form series against closed forms and its own
finite differences; the package's W_krivanek / grad_W_krivanek against the
oracle; the host float64 ABCD through an AberratedLensKrivanek (monomial
Hessian) against the oracle's finite-difference Jacobian.  No reference KATs
exist for this component, so parity is pinned by the closed forms."""
import numpy as np

from oracle import rays as OR

COEF_NAMES = OR._KRIV


def _random_coeffs(rng, f=0.2, alpha=2e-3):
    """Coefficients scaled so every order kicks the slope by ~10% of alpha."""
    c = {}
    for n in COEF_NAMES:
        if n.startswith("phi"):
            c[n] = float(rng.uniform(-np.pi, np.pi))
        else:
            order = int(n[1])  # C_{n-1, m}: W ~ C alpha^(order+1)
            c[n] = float(rng.normal(0.0, 0.1 * f / alpha ** (order - 1) / (order + 1)))
    return c


def test_closed_forms():
    rng = np.random.default_rng(0)
    ax, ay = rng.normal(0, 1e-3, 50), rng.normal(0, 1e-3, 50)
    a, ph = np.hypot(ax, ay), np.arctan2(ay, ax)
    # defocus C10: W = C10 a^2 / 2, grad = C10 (ax, ay)
    gx, gy = OR.grad_w_krivanek(ax, ay, {"C10": 3.0})
    np.testing.assert_allclose(OR.w_krivanek(a, ph, {"C10": 3.0}), 1.5 * a ** 2, rtol=1e-14)
    np.testing.assert_allclose(gx, 3.0 * ax, rtol=1e-12)
    np.testing.assert_allclose(gy, 3.0 * ay, rtol=1e-12)
    # spherical C30: W = C30 a^4 / 4, grad = C30 a^2 (ax, ay)
    gx, gy = OR.grad_w_krivanek(ax, ay, {"C30": 5e4})
    np.testing.assert_allclose(OR.w_krivanek(a, ph, {"C30": 5e4}), 1.25e4 * a ** 4, rtol=1e-13)
    np.testing.assert_allclose(gx, 5e4 * a ** 2 * ax, rtol=1e-12)
    # two-fold astigmatism C12, phi12 = 0: W = C12 (ax^2 - ay^2) / 2
    gx, gy = OR.grad_w_krivanek(ax, ay, {"C12": 2.0})
    np.testing.assert_allclose(OR.w_krivanek(a, ph, {"C12": 2.0}), ax ** 2 - ay ** 2, rtol=1e-12, atol=1e-22)
    np.testing.assert_allclose(gx, 2.0 * ax, rtol=1e-11)
    np.testing.assert_allclose(gy, -2.0 * ay, rtol=1e-11)
    # alpha = 0: zero gradient (the reference's guarded division)
    gx, gy = OR.grad_w_krivanek(np.zeros(1), np.zeros(1), _random_coeffs(rng))
    assert gx[0] == 0.0 and gy[0] == 0.0


def test_gradient_is_derivative_of_w():
    rng = np.random.default_rng(1)
    c = _random_coeffs(rng)
    ax, ay = rng.normal(0, 2e-3, 40), rng.normal(0, 2e-3, 40)
    h = 1e-8
    W = lambda u, v: OR.w_krivanek(np.hypot(u, v), np.arctan2(v, u), c)  # noqa: E731
    fdx = (W(ax + h, ay) - W(ax - h, ay)) / (2 * h)
    fdy = (W(ax, ay + h) - W(ax, ay - h)) / (2 * h)
    gx, gy = OR.grad_w_krivanek(ax, ay, c)
    scale = np.max(np.abs(np.concatenate([gx, gy])))
    assert np.max(np.abs(gx - fdx)) / scale < 1e-6
    assert np.max(np.abs(gy - fdy)) / scale < 1e-6


def test_package_series_matches_oracle():
    import torch

    from temgymcore_gb300.aberrations import KrivanekCoeffs, W_krivanek, grad_W_krivanek
    rng = np.random.default_rng(2)
    c = _random_coeffs(rng)
    ax, ay = rng.normal(0, 2e-3, 64), rng.normal(0, 2e-3, 64)
    a, ph = np.hypot(ax, ay), np.arctan2(ay, ax)
    kc = KrivanekCoeffs(**c)
    np.testing.assert_allclose(W_krivanek(a, ph, kc), OR.w_krivanek(a, ph, c), rtol=1e-12, atol=1e-30)
    for got, ref in zip(grad_W_krivanek(ax, ay, kc), OR.grad_w_krivanek(ax, ay, c)):
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-30)
    tx, ty = torch.tensor(ax), torch.tensor(ay)
    for got, ref in zip(grad_W_krivanek(tx, ty, c), OR.grad_w_krivanek(ax, ay, c)):
        np.testing.assert_allclose(got.numpy(), ref, rtol=1e-12, atol=1e-30)


def test_brackets_and_zero_slope_match_oracle():
    from oracle.rays import _brackets, _kc
    from temgymcore_gb300.aberrations import KrivanekCoeffs, grad_W_krivanek, krivanek_coeff_brackets
    rng = np.random.default_rng(4)
    c = _random_coeffs(rng)
    ph = rng.uniform(-np.pi, np.pi, 32)
    ref = _brackets(ph, _kc(c))
    got = krivanek_coeff_brackets(ph, KrivanekCoeffs(**c))
    for g, r in zip(got, ref):
        np.testing.assert_allclose(g, r, rtol=1e-12, atol=1e-12 * np.max(np.abs(r)))
    gx, gy = grad_W_krivanek(np.zeros(3), np.zeros(3), KrivanekCoeffs(**c))
    assert np.all(gx == 0) and np.all(gy == 0)  # the reference's alpha = 0 guard gives 0 too


def test_host_abcd_through_aberrated_lens():
    import oracle
    import temgymcore_gb300 as T
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(3)
    spec = [{"kind": "lens", "z": 0.1, "focal_length": 0.5},
            {"kind": "aberrated_lens", "z": 0.3, "focal_length": 0.2, "coeffs": _random_coeffs(rng)},
            {"kind": "deflector", "z": 0.4, "def_x": 1e-4, "def_y": -2e-4},
            {"kind": "detector", "z": 0.6, "pixel_size": (1e-5, 1e-5), "shape": (64, 64)}]
    for cen in ((1e-4, -2e-4, 1.5e-3, 1e-3, 0.0), (0.0, 0.0, 0.0, 0.0, 0.0), (-3e-4, 1e-4, -1e-3, 2e-3, 0.0)):
        ref = oracle.model_abcd(ORay(*cen[:4], z=cen[4], pathlength=0.0), spec)
        got = T.abcd_matrix(T.Ray(*cen, pathlength=0.0), build_model(spec))
        # the oracle's Hessian is a central difference (~1e-9 relative)
        np.testing.assert_allclose(got, ref, rtol=1e-7, atol=1e-9 * np.abs(ref).max())
