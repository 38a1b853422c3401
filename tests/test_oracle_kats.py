"""The oracle against the reference's own known answers (CPU only)."""
import numpy as np
import pytest

import oracle
from oracle.rays import ORay, accumulate_matrices, free_matrix, component_matrix
from oracle import field as OF


def _ray(v):
    return ORay(*v[:4], z=v[4], pathlength=v[5])


def test_readme_quickstart(kats):
    q = kats["readme_quickstart"]
    r = q["ray"]
    o = oracle.run_to_end(ORay(r["x"], r["y"], r["dx"], r["dy"], r["z"], r["pathlength"]), q["model"])
    e = q["expected"]
    for k in ("x", "y", "dx", "dy", "z", "pathlength"):
        assert abs(float(getattr(o, k)) - e[k]) < 1e-12, k
    assert abs(float(o.pathlength) - q["printed_pathlength"]) < 0.005


def test_readme_abcd_and_steps(kats):
    q = kats["readme_quickstart"]
    r = q["ray"]
    ray = ORay(r["x"], r["y"], r["dx"], r["dy"], r["z"], r["pathlength"])
    np.testing.assert_allclose(oracle.model_abcd(ray, q["model"]), kats["readme_abcd"]["abcd"], atol=1e-15)
    steps = oracle.solve_model(ray, q["model"])
    np.testing.assert_allclose(steps, kats["readme_abcd"]["per_step"], atol=1e-15)


def test_readme_grads_by_complex_step(kats):
    q = kats["readme_quickstart"]
    r = q["ray"]
    h = 1e-30
    # d x_out / d f  and  d x_out / d z_lens
    m = [dict(q["model"][0], focal_length=1.0 + 1j * h), q["model"][1]]
    o = oracle.run_to_end(ORay(r["x"], r["y"], r["dx"], r["dy"], r["z"], r["pathlength"]), m)
    gf = np.imag(o.x) / h
    m = [dict(q["model"][0], z=0.5 + 1j * h), q["model"][1]]
    o = oracle.run_to_end(ORay(r["x"], r["y"], r["dx"], r["dy"], r["z"], r["pathlength"]), m)
    gz = np.imag(o.x) / h
    np.testing.assert_allclose([gf, gz], kats["readme_grads"]["dx_out_d_f_and_z"], rtol=1e-12)
    o = oracle.run_to_end(ORay(0.01 + 1j * h, 0.2, 0.3, 0.4, 0.0, 0.6), q["model"])
    assert abs(np.imag(o.dx) / h - kats["readme_grads"]["ddx_out_dx_in"]) < 1e-12
    assert abs(np.imag(o.dy) / h - kats["readme_grads"]["ddy_out_dx_in"]) < 1e-12


def test_pixel_kats(kats):
    for (xy, rot, exp) in kats["scangrid_m2p"]["cases"]:
        g = {"pixel_size": (0.1, 0.1), "shape": (11, 11), "rotation": rot}
        assert tuple(int(v) for v in oracle.metres_to_pixels(g, xy[0], xy[1])) == tuple(exp)
    for (px, rot, exp) in kats["scangrid_p2m"]["cases"]:
        g = {"pixel_size": (0.1, 0.1), "shape": (11, 11), "rotation": rot}
        np.testing.assert_allclose(oracle.pixels_to_metres(g, px[0], px[1]), exp, atol=1e-6)
    for (xy, exp) in kats["detector_m2p"]["cases"]:
        g = {"pixel_size": (0.1, 0.1), "shape": (11, 11)}
        assert tuple(int(v) for v in oracle.metres_to_pixels(g, xy[0], xy[1])) == tuple(exp)
    for (px, exp) in kats["detector_p2m"]["cases"]:
        g = {"pixel_size": (0.1, 0.1), "shape": (11, 11)}
        np.testing.assert_allclose(oracle.pixels_to_metres(g, px[0], px[1]), exp, atol=1e-6)


@pytest.mark.parametrize("shape", [(5, 5), (3, 7), (4, 4), (5, 8)])
def test_scangrid_symmetry(shape):
    h, w = shape
    g = {"pixel_size": (0.1, 0.1), "shape": shape}
    _, yv = oracle.pixels_to_metres(g, np.arange(h), np.zeros(h))
    xv, _ = oracle.pixels_to_metres(g, np.zeros(w), np.arange(w))
    for size, v in ((h, yv), (w, xv)):
        if size % 2 == 0:
            assert np.count_nonzero(v) == size
            assert v[size // 2] == pytest.approx(-v[size // 2 - 1])
        else:
            assert np.count_nonzero(v) == size - 1
            assert v[size // 2] == pytest.approx(0.0)


def test_scanner_descanner_formulas(kats):
    for c in kats["scanner"]["cases"]:
        spx, spy, stx, sty = c["scanner"]
        o = oracle.apply_component({"kind": "scanner", "z": 23, "scan_pos_x": spx, "scan_pos_y": spy,
                                    "scan_tilt_x": stx, "scan_tilt_y": sty}, _ray(c["ray"]))
        np.testing.assert_allclose([o.x, o.y, o.dx, o.dy], c["expected"], atol=1e-12)
    for c in kats["descanner"]["cases"]:
        spx, spy, stx, sty = c["scan"]
        o = oracle.apply_component({"kind": "descanner", "z": 23, "scan_pos_x": spx, "scan_pos_y": spy,
                                    "scan_tilt_x": stx, "scan_tilt_y": sty,
                                    "descan_error": c["err"]}, _ray(c["ray"]))
        np.testing.assert_allclose([o.x, o.y, o.dx, o.dy], c["expected"], atol=1e-12)
    d = kats["descanner_jacobian"]
    m = component_matrix({"kind": "descanner", "z": 0.0, "scan_pos_x": d["scan"][0],
                          "scan_pos_y": d["scan"][1], "descan_error": d["err"]})
    np.testing.assert_allclose(m, d["expected"], atol=1e-12)


def test_biprism_and_chain(kats):
    b = kats["biprism"]
    m = component_matrix({"kind": "biprism", "z": 0.0, "def_x": b["deflection"]}, 1e-15)
    assert abs(m[2, 4] - b["jac_dx_one"]) < 1e-12
    model = [{"kind": "biprism", "z": 0.0, "def_x": b["deflection"]},
             {"kind": "detector", "z": b["z_det"], "pixel_size": (1e-4, 1e-4), "shape": (512, 512)}]
    a = oracle.model_abcd(ORay(1e-15, 0.0, 0.0, 0.0, 0.0, 0.0), model)
    assert abs(a[0, 4] - b["prop_x_one"]) < 1e-12 and abs(a[2, 4] - b["prop_dx_one"]) < 1e-12
    c = kats["lens_biprism_chain"]
    cr = c["central_ray"]
    a = oracle.model_abcd(ORay(cr["x"], cr["y"], cr["dx"], cr["dy"], cr["z"], 0.0), c["model"])
    np.testing.assert_allclose(a, c["abcd"], atol=c["atol"])


def test_propagation_and_run_iter(kats):
    for c in kats["propagation"]["cases"]:
        o = oracle.propagate(_ray(c["ray"]), c["d"])
        np.testing.assert_allclose([o.x, o.y, o.dx, o.dy, o.z, o.pathlength], c["expected"], atol=1e-12)
        np.testing.assert_allclose(free_matrix(c["d"])[0, 2], c["d"])
    ri = kats["run_iter"]
    res = list(oracle.run_iter(_ray(ri["ray"]), ri["model"]))
    prev = _ray(ri["ray"])
    for i, comp in enumerate(ri["model"]):
        (_, d), pr = res[2 * i]
        assert d == comp["z"] - prev.z
        np.testing.assert_allclose(pr.x, prev.x + prev.dx * d)
        prev = res[2 * i + 1][1]
    # no-propagation case equals composing the components directly
    r0 = _ray(ri["noprop_ray"])
    out = oracle.run_to_end(r0, ri["noprop_model"])
    ref = r0
    for comp in ri["noprop_model"]:
        ref = oracle.apply_component(comp, ref)
    for k in ("x", "y", "dx", "dy", "z", "pathlength"):
        np.testing.assert_allclose(getattr(out, k), getattr(ref, k))


def test_accumulate_order(kats):
    mats = []
    for s in kats["accumulate"]["scales"]:
        m = np.eye(5) * s
        m[4] = [0, 0, 0, 0, 1]
        mats.append(m)
    np.testing.assert_allclose(accumulate_matrices(mats), mats[2] @ mats[1] @ mats[0])


def test_gauss_free_space_closed_form(kats):
    g = kats["gauss_free_space"]
    wl, w0, L = g["wavelength"], g["w0"], g["L"]
    k = 2 * np.pi / wl
    q = 1j * wl / (np.pi * w0 * w0)
    q1 = np.array([[[q, 0], [0, q]]], dtype=np.complex128)
    A = np.array([np.eye(2)])
    B = np.array([L * np.eye(2)])
    C = np.zeros((1, 2, 2))
    D = np.array([np.eye(2)])
    q2 = OF.Qinv_ABCD(q1, A, B, C, D)
    f = OF.beam_field_pixels(np.array([1.0 + 0j]), np.array([0.0]), q1, q2, np.zeros((1, 2)),
                             np.zeros((1, 2)), A, B, np.zeros((1, 2)), np.zeros((1, 2)),
                             np.array([k]), np.array(g["r2"]))[0]
    ref = np.array(g["field_re"]) + 1j * np.array(g["field_im"])
    np.testing.assert_allclose(f, ref, rtol=g["rtol"], atol=g["atol"])
    # Qinv_ABCD identity (tests/test_gaussians.py:218-226)
    q1 = np.array([[[2j, 0], [0, 3j]]])
    np.testing.assert_allclose(OF.Qinv_ABCD(q1, A, np.zeros((1, 2, 2)), C, D), q1, rtol=1e-12)


def test_gauss_profile_helpers():
    """zR, w_z, R, q_inv(z, w0, wl) and gaussian_beam against their closed
    forms (tests/test_gaussians.py:167-214: 1 mm waist, 500 nm)."""
    w0, wl = 1e-3, 500e-9
    zr = float(OF.zR(w0, wl))
    assert np.isclose(zr, np.pi * w0 * w0 / wl, rtol=1e-9, atol=0)
    assert np.isclose(OF.w_z(w0, 0.0, zr), w0, rtol=1e-9, atol=0)
    assert np.isclose(OF.w_z(w0, zr, zr), w0 * np.sqrt(2.0), rtol=1e-9, atol=0)
    assert np.isclose(OF.R_of_z(zr, zr), 2 * zr, rtol=1e-9, atol=0) and np.isinf(OF.R_of_z(0.0, zr))
    assert np.allclose(OF.q_inv_z(0.0, w0, wl), 1j * wl / (np.pi * w0 * w0), rtol=1e-12, atol=0)
    exp = -(1.0 / (2 * zr)) + 1j * wl / (np.pi * (w0 * np.sqrt(2.0)) ** 2)
    assert np.allclose(OF.q_inv_z(zr, w0, wl), exp, rtol=1e-12, atol=0)
    k = 2 * np.pi / wl
    assert np.allclose(OF.gaussian_beam(0.0, 0.0, 1j * 1e-6, k), 1.0, rtol=1e-12, atol=0)
    assert np.allclose(OF.gaussian_beam(1e-3, -2e-3, 1j * 1e-6, k, offset_x=-1e-3, offset_y=2e-3), 1.0,
                       rtol=1e-12, atol=0)
    # the per-beam q_inv at a waist (R = inf) is q_inv(0, w0, wl)
    qx, qy = OF.q_inv(np.array([[w0, 2 * w0]]), np.array([[np.inf, np.inf]]), wl)
    assert np.allclose(qx, OF.q_inv_z(0.0, w0, wl), rtol=1e-15) and np.allclose(
        qy, OF.q_inv_z(0.0, 2 * w0, wl), rtol=1e-15)


def test_gauss_quadrant(kats):
    g = kats["gauss_quadrant"]
    det = {"kind": "detector", "z": g["z"], "pixel_size": g["pixel_size"], "shape": g["shape"]}
    xs, ys = np.meshgrid(*[np.arange(s) for s in g["shape"][::-1]])
    c = OF.make_gaussian_image({"x": 0.0, "y": 0.0, "dx": 0.0, "dy": 0.0, "z": 0.0, "pathlength": 0.0,
                                "amplitude": 1.0, "waist_xy": [[g["w0"], g["w0"]]],
                                "radii_of_curv": [[np.inf, np.inf]], "wavelength": g["wavelength"],
                                "theta": 0.0}, [det])
    cy, cx = np.unravel_index(np.argmax(np.abs(c)), c.shape)
    xc, yc = oracle.pixels_to_metres(det, cy, cx)
    t = g["tilt"]
    for dx, dy in ((t, t), (t, -t), (-t, t), (-t, -t)):
        im = OF.make_gaussian_image({"x": 0.0, "y": 0.0, "dx": dx, "dy": dy, "z": 0.0, "pathlength": 0.0,
                                     "amplitude": 1.0, "waist_xy": [[g["w0"], g["w0"]]],
                                     "radii_of_curv": [[np.inf, np.inf]],
                                     "wavelength": g["wavelength"], "theta": 0.0}, [det])
        my, mx = np.unravel_index(np.argmax(np.abs(im)), im.shape)
        xm, ym = oracle.pixels_to_metres(det, my, mx)
        assert np.sign(xm - xc) == np.sign(dx) and np.sign(ym - yc) == np.sign(dy)


def test_phase_reduction_exact():
    rng = np.random.default_rng(3)
    k = 2 * np.pi / 1.97e-12
    pl = 1.0 + rng.normal(0, 1e-6, 64)
    red = oracle.phase_offset_exact(k, pl)
    # cross-check against extended precision (x86 80-bit here; 128-bit on Arm)
    ld = np.longdouble
    exact = (ld(k) * pl.astype(ld))
    twopi = ld("6.283185307179586476925286766559")
    ref = exact - np.rint(exact / twopi) * twopi
    err = np.abs(np.angle(np.exp(1j * (red - ref.astype(np.float64)))))
    assert err.max() < 1e-6
    # the literal float64 product is off by up to ~ulp(3e12) / 2 ~ 2.4e-4 rad
    lit = np.angle(np.exp(1j * (k * pl)))
    assert np.abs(np.angle(np.exp(1j * (lit - red)))).max() > 1e-6


def _one_beam(x0, y0, dx, dy, wavelength=500e-9, w0=1e-4, theta=0.0, waist=None):
    return {"x": np.array([x0]), "y": np.array([y0]), "dx": np.array([dx]), "dy": np.array([dy]),
            "z": 0.0, "pathlength": np.array([0.0]), "amplitude": np.array([1.0 + 0j]),
            "waist_xy": np.array([[w0, w0]] if waist is None else [waist]),
            "radii_of_curv": np.array([[np.inf, np.inf]]), "wavelength": wavelength,
            "theta": np.array([theta])}


def test_oracle_input_field_phase_ramp():
    """tests/test_gaussians.py:736-786: the input-plane field of a tilted beam
    has zero phase at its centre and a phase slope k * tilt."""
    from oracle import field as OF
    from oracle.grid import grid_coords
    det = {"kind": "detector", "z": 0.0, "pixel_size": (1e-5, 1e-5), "shape": (512, 512)}
    xy = grid_coords(det).reshape(512, 512, 2)
    det_x, det_y = xy[0, :, 0], xy[:, 0, 1]
    ix = iy = 256
    wl = 500e-9
    k = 2 * np.pi / wl
    for dx, dy in ((2e-4, 0.0), (0.0, -1e-4), (1.5e-4, -1.0e-4)):
        img = OF.evaluate_gaussian_input_image(_one_beam(det_x[ix], det_y[iy], dx, dy, wl), det)
        assert abs(np.angle(img[iy, ix])) < 1e-6
        rp = np.unwrap(np.angle(img[iy, :]))
        cp = np.unwrap(np.angle(img[:, ix]))
        sx = (rp[ix + 8] - rp[ix - 8]) / (det_x[ix + 8] - det_x[ix - 8])
        sy = (cp[iy + 8] - cp[iy - 8]) / (det_y[iy + 8] - det_y[iy - 8])
        np.testing.assert_allclose(sx, k * dx, rtol=2e-2, atol=1e-3)
        np.testing.assert_allclose(sy, k * dy, rtol=2e-2, atol=1e-3)


def _principal_axis_angle(field, X, Y):
    intensity = np.abs(field) ** 2
    w = intensity.sum() + 1e-30
    xb, yb = (intensity * X).sum() / w, (intensity * Y).sum() / w
    cxx = (intensity * (X - xb) ** 2).sum() / w
    cyy = (intensity * (Y - yb) ** 2).sum() / w
    cxy = (intensity * (X - xb) * (Y - yb)).sum() / w
    vals, vecs = np.linalg.eigh(np.array([[cxx, cxy], [cxy, cyy]]))
    v = vecs[:, np.argmax(vals)]
    return (np.arctan2(v[1], v[0]) + np.pi / 2) % np.pi - np.pi / 2


def test_oracle_input_field_astigmatic_rotation():
    """tests/test_gaussians.py:818-877: the major axis of an astigmatic input
    beam follows theta."""
    from oracle import field as OF
    from oracle.grid import grid_coords
    det = {"kind": "detector", "z": 0.0, "pixel_size": (1e-5, 1e-5), "shape": (512, 512)}
    xy = grid_coords(det).reshape(512, 512, 2)
    X, Y = xy[..., 0], xy[..., 1]
    for th in (np.pi / 3, np.pi / 6, 0.0, -np.pi / 6, -np.pi / 3, -np.pi / 2 + 0.1):
        img = OF.evaluate_gaussian_input_image(_one_beam(0.0, 0.0, 0.0, 0.0, theta=th,
                                                         waist=[2e-4, 1e-4]), det)
        phi = _principal_axis_angle(img, X, Y)
        assert abs(np.arctan2(np.sin(phi - th), np.cos(phi - th))) < 0.1


def _fresnel_case(model, wavelength, w0, fresnel):
    """The oracle's single-beam field against a Fresnel FFT propagation of
    the same Gaussian input (tests/test_gaussians.py:276-519): both
    normalised to unit peak and to zero phase at the centre pixel, compared
    inside a disc of 0.4 of the half-width."""
    from oracle.grid import grid_coords
    det = model[-1]
    h, w = det["shape"]
    rays = {"x": 0.0, "y": 0.0, "dx": 0.0, "dy": 0.0, "z": 0.0, "pathlength": 0.0, "amplitude": 1.0,
            "waist_xy": [[w0, w0]], "radii_of_curv": [[np.inf, np.inf]], "wavelength": wavelength,
            "theta": 0.0}
    a = OF.make_gaussian_image(rays, model, chunk=1)
    xy = grid_coords(det)
    X, Y = xy[:, 0].reshape(h, w), xy[:, 1].reshape(h, w)
    g = OF.gaussian_beam(X, Y, OF.q_inv_z(0.0, w0, wavelength), 2 * np.pi / wavelength)
    b = fresnel(g, X, Y)
    out = []
    for u in (a, b):
        u = u * np.exp(-1j * np.angle(u[h // 2, w // 2]))
        out.append(u / np.max(np.abs(u)))
    mask = (X ** 2 + Y ** 2) < (0.4 * np.max(np.abs(X))) ** 2
    amp = np.max(np.abs(np.abs(out[0][mask]) - np.abs(out[1][mask])))
    ph = np.abs(np.angle(out[0][mask] * np.conj(out[1][mask])))
    return amp, ph.max()


def test_oracle_free_space_vs_fresnel():
    d, px, n, wl, w0 = 1e-3, 5e-4, 2000, 1e-3, 0.1
    model = [{"kind": "source", "z": 0.0},
             {"kind": "detector", "z": d, "pixel_size": (px, px), "shape": (n, n)}]
    amp, ph = _fresnel_case(model, wl, w0, lambda g, X, Y: OF.fresnel_tf(g, n * px, wl, d))
    assert amp <= 1e-1 and ph <= 1e-1, (amp, ph)


def test_oracle_lens_vs_fresnel():
    """M = -2 imaging with f = 5 mm and 0.1 mm defocus (z1, z2 from the thin
    lens equation, tests/transfer_matrices.py:263-271)."""
    M, f, defocus, px, n, wl, w0 = -2.0, 5e-3, 1e-4, 5e-6, 2048, 1e-5, 5e-4
    z1, z2 = f * (1 / M - 1), f * (1 - M)
    model = [{"kind": "source", "z": 0.0},
             {"kind": "lens", "z": abs(z1) + defocus, "focal_length": f},
             {"kind": "detector", "z": abs(z1) + z2, "pixel_size": (px, px), "shape": (n, n)}]
    amp, ph = _fresnel_case(model, wl, w0,
                            lambda g, X, Y: OF.fresnel_thin_lens(g, X, Y, px, wl, defocus + abs(z1), f, z2))
    assert amp <= 5e-1 and ph <= 2.0, (amp, ph)


def test_oracle_two_beam_interference_vs_fresnel():
    """Two beams tilted 0.1 rad (in y and in x) through a 5 mm lens to 2 mm
    past focus, against the Fresnel FFT of the summed tilted Gaussians
    (tests/test_gaussians.py:520-681).  Normalised to unit peak and zero
    centre phase; amplitudes compared inside 0.8 of the half-width (the
    reference's 0.5), phases at pixels above a quarter of the peak."""
    from oracle.grid import grid_coords
    px, n, f, defocus, wl, w0 = 5e-6, 1024, 5e-3, 2e-3, 1e-4, 0.5e-3
    z2 = f + defocus
    det = {"kind": "detector", "z": z2, "pixel_size": (px, px), "shape": (n, n)}
    model = [{"kind": "lens", "z": 0.0, "focal_length": f}, det]
    tilts = [(0.0, 0.1), (0.1, 0.0)]  # (dx, dy)
    rays = {"x": np.zeros(2), "y": np.zeros(2), "dx": np.array([t[0] for t in tilts]),
            "dy": np.array([t[1] for t in tilts]), "z": 0.0, "pathlength": np.zeros(2),
            "amplitude": np.ones(2), "waist_xy": np.full((2, 2), w0), "radii_of_curv": np.full((2, 2), np.inf),
            "wavelength": wl, "theta": np.zeros(2)}
    a = OF.make_gaussian_image(rays, model, chunk=1)
    xy = grid_coords(det)
    X, Y = xy[:, 0].reshape(n, n), xy[:, 1].reshape(n, n)
    k = 2 * np.pi / wl
    g = sum(OF.gaussian_beam(X, Y, OF.q_inv_z(0.0, w0, wl), k) * np.exp(1j * k * (X * tx + Y * ty))
            for tx, ty in tilts)
    b = OF.fresnel_thin_lens(g, X, Y, px, wl, 0.0, f, z2)
    out = []
    for u in (a, b):
        u = u * np.exp(-1j * np.angle(u[n // 2, n // 2]))
        out.append(u / np.max(np.abs(u)))
    mask = (X ** 2 + Y ** 2) < (0.8 * np.max(np.abs(X))) ** 2
    amp = np.max(np.abs(np.abs(out[0][mask]) - np.abs(out[1][mask])))
    bright = mask & (np.abs(out[1]) > 0.25)
    ph = np.max(np.abs(np.angle(out[0][bright] * np.conj(out[1][bright]))))
    assert amp <= 5e-1 and ph <= 2.0, (amp, ph)


def test_oracle_input_slope_and_angle_vs_fresnel():
    """A beam with a random offset and tilt: the peak of its detector field at
    1 m is where the Fresnel FFT of its input-plane field peaks, within 3
    pixels of flat index (tests/test_gaussians.py:788-817; seeded here)."""
    rng = np.random.default_rng(7)
    n, px, z, wl = 1024, 1e-5, 1.0, 500e-9
    det = {"kind": "detector", "z": z, "pixel_size": (px, px), "shape": (n, n)}
    for _ in range(3):
        r1m = rng.uniform(-1e-3, 1e-3, 2)
        t1m = rng.uniform(-1e-4, 1e-4, 2)
        rays = {"x": r1m[0], "y": r1m[1], "dx": t1m[0], "dy": t1m[1], "z": 0.0, "pathlength": 0.0,
                "amplitude": 1.0, "waist_xy": [[1e-4, 1e-4]], "radii_of_curv": [[np.inf, np.inf]],
                "wavelength": wl, "theta": 0.0}
        inp = OF.evaluate_gaussian_input_image(rays, dict(det, z=0.0), chunk=1)
        out = OF.make_gaussian_image(rays, [det], chunk=1)
        fr = OF.fresnel_tf(inp, n * px, wl, z)
        assert abs(int(np.argmax(np.abs(fr))) - int(np.argmax(np.abs(out)))) <= 3
