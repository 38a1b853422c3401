"""Host-side logic of the package (CPU only): record packing, sizes,
pixel maps, workload generators, gradient mapping."""
import numpy as np
import torch

import oracle


def test_gaussian_ray_size_and_beamset():
    from temgymcore_gb300 import GaussianRay
    from temgymcore_gb300.gaussian import BeamSet, pixel_map
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    w = beamlet_field(seed=0, n_beams=100, det_shape=(32, 48))
    r = gaussian_rays(w["rays"])
    assert r.size == 100
    b = BeamSet(r, torch.device("cpu"))
    assert b.n == 100 and b.waist.shape == (100, 2) and b.amp.shape == (100, 2)
    assert b.wl.shape == (100,) and b.theta.shape == (100,) and b.z == 0.0
    g = GaussianRay(x=0.0, y=0.0, dx=0.0, dy=0.0, z=0.0, pathlength=0.0, amplitude=1.0,
                    waist_xy=np.array([1e-4, 2e-4]), radii_of_curv=np.array([np.inf, np.inf]),
                    wavelength=5e-7, theta=0.0)
    assert g.size == 1
    det = build_model(w["model"])[-1]
    pm = pixel_map(det)
    t = oracle.pixels_to_metres_transform((0.0, 0.0), det.pixel_size, det.shape)
    assert (pm.h, pm.w) == (32, 48)
    np.testing.assert_array_equal(list(pm.t), [t[0, 0], t[0, 1], t[0, 2], t[1, 0], t[1, 1], t[1, 2]])


def test_fibonacci_and_transforms_match_oracle():
    from temgymcore_gb300 import fibonacci_spiral, Detector
    from oracle.field import fibonacci_spiral as ofs
    for a in (0, 2):
        np.testing.assert_array_equal(np.array(fibonacci_spiral(1000, 1e-7, a)), np.array(ofs(1000, 1e-7, a)))
    det = Detector(z=0.0, pixel_size=(2e-5, 1e-5), shape=(100, 300), rotation=33.0,
                   centre=(1e-4, -3e-4), flip_y=True)
    g = {"pixel_size": (2e-5, 1e-5), "shape": (100, 300), "rotation": 33.0,
         "centre": (1e-4, -3e-4), "flip_y": True}
    np.testing.assert_array_equal(det.metres_to_pixels_mat,
                                  oracle.metres_to_pixels_mat(g["centre"], g["pixel_size"], g["shape"],
                                                              True, 33.0))
    np.testing.assert_array_equal(det.coords, oracle.grid_coords(g))


def test_pack_model_records():
    import ctypes
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.run import pack_model
    from temgymcore_gb300.workloads import build_model
    spec = [{"kind": "lens", "z": 0.5, "focal_length": 0.2},
            {"kind": "descanner", "z": 0.6, "scan_pos_x": 1.0, "scan_pos_y": 2.0,
             "descan_error": {"pxo_pxi": 3.0, "offsyi": 4.0, "syo_syi": 5.0}},
            {"kind": "thicklens", "z_po": 0.7, "z_pi": 0.8, "focal_length": 0.1},
            {"kind": "aperture", "z": 0.9, "radius": 1e-3, "centre": (1e-4, 2e-4)},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (8, 8)}]
    m, keep = pack_model(build_model(spec))
    c = [m.components[i] for i in range(m.n_components)]
    assert [x.kind for x in c] == [N.LENS, N.DESCANNER, N.THICKLENS, N.APERTURE, N.PLANE]
    assert c[0].p[0] == 0.2 and c[2].z == 0.7 and c[2].p[1] == 0.8
    assert c[1].p[0] == 1.0 and c[1].p[4] == 3.0 and c[1].p[23] == 4.0 and c[1].p[4 + 15] == 5.0
    assert c[3].p[0] == 1e-3 and c[3].p[1] == 1e-4 and c[3].p[2] == 2e-4


def test_param_gradient_mapping_descanner():
    """dL/dparams from per-step adjoint sums: checked against the chain rule
    on the oracle's descanner offsets."""
    from temgymcore_gb300.run import param_gradient
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(2)
    err = dict(zip(["pxo_pxi", "pxo_pyi", "pyo_pxi", "pyo_pyi", "sxo_pxi", "sxo_pyi", "syo_pxi",
                    "syo_pyi", "offpxi", "offpyi", "offsxi", "offsyi"], rng.normal(0, 1, 12)))
    spec = [{"kind": "descanner", "z": 0.0, "scan_pos_x": 0.3, "scan_pos_y": -0.2,
             "scan_tilt_x": 0.1, "scan_tilt_y": 0.05, "descan_error": err}]
    comps = build_model(spec)
    g = rng.normal(0, 1, 4)  # dL/d(delta x, delta y, delta dx, delta dy)
    raw = torch.zeros((2, 4), dtype=torch.float64)
    raw[1] = torch.tensor(g)
    h = 1e-30
    for path in ("scan_pos_x", "scan_pos_y", "scan_tilt_x", "scan_tilt_y",
                 "descan_error.pxo_pxi", "descan_error.syo_pyi", "descan_error.offsxi"):
        s = [dict(c) for c in spec]
        if path.startswith("descan"):
            e = dict(s[0]["descan_error"])
            e[path.split(".")[1]] += 1j * h
            s[0]["descan_error"] = e
        else:
            s[0][path] = s[0][path] + 1j * h
        o = oracle.apply_component(s[0], oracle.ORay(0.0, 0.0, 0.0, 0.0, 0.0, 0.0))
        ref = sum(gi * np.imag(getattr(o, k)) / h for gi, k in zip(g, ("x", "y", "dx", "dy")))
        assert abs(float(param_gradient(comps, 0, path, raw)) - ref) < 1e-12 * max(1, abs(ref))


def test_workloads_are_seeded():
    from temgymcore_gb300.workloads import plain_trace, stem_4d, beamlet_field
    a, b = plain_trace(seed=0, n=100), plain_trace(seed=0, n=100)
    assert np.array_equal(a["x"], b["x"]) and a["x"].dtype == np.float32
    s = stem_4d(seed=0)
    assert s["dx"].shape == (1024,) and 0.0 <= s["scangrid"]["rotation"] < 360.0
    f = beamlet_field(seed=0, n_beams=16)
    assert f["rays"]["amplitude"].dtype == np.complex64


def test_path_builder_and_custom_jacobian_matrix():
    """PathBuilder paths (tree_utils.py:34-122) and custom_jacobian_matrix
    (utils.py:7-43) on the host."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.run import _param_paths, _ray_of_rays
    from temgymcore_gb300.utils import custom_jacobian_matrix
    lens = t.Lens(z=0.5, focal_length=0.2)
    p = lens.params.focal_length
    assert p._build() == (lens, "focal_length") and p._resolve() == 0.2 and p._resolve_root() is lens
    d = t.Descanner(z=1.0, scan_pos_x=0.0, scan_pos_y=0.0, scan_tilt_x=0.0, scan_tilt_y=0.0)
    q = d.params.descan_error.offsxi
    assert q._build() == (d, "descan_error", "offsxi")
    assert _param_paths(d, ("descan_error",)) == ["descan_error." + f for f in t.DescanError._fields]
    assert _param_paths(d, ("descan_error", "offsxi")) == ["descan_error.offsxi"]
    assert _param_paths(lens, ("focal_length",)) == ["focal_length"]
    assert _param_paths(lens, ("nonexistent",)) == []
    r = t.Ray(x=0.1, y=0.2, dx=0.3, dy=0.4, z=0.0, pathlength=0.0)
    assert r.params._one._build() == (r, "_one")
    m = np.arange(25, dtype=np.float64).reshape(5, 5)
    np.testing.assert_array_equal(custom_jacobian_matrix(_ray_of_rays(m)), m)


def test_apply_transformation_and_descan_matrix():
    """apply_transformation (coordinate_transforms.py:104-140) and
    DescanError.as_matrix (components.py:93-115) on the host."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.coordinate_transforms import apply_transformation
    y, x = np.array([0.0, 1.0]), np.array([2.0, 3.0])
    y2, x2 = apply_transformation(y, x, np.eye(3))
    assert np.array_equal(y2, y) and np.array_equal(x2, x)
    det = t.Detector(z=0.0, pixel_size=(0.1, 0.1), shape=(11, 11))
    py, px = apply_transformation(np.array([0.0, 5.0]), np.array([0.0, 5.0]), det.metres_to_pixels_mat)
    np.testing.assert_allclose(py, [5.0, -45.0]) and np.testing.assert_allclose(px, [5.0, 55.0])
    e = t.DescanError(*range(1, 13))
    m = e.as_matrix()
    assert m.shape == (5, 5) and m[0, 4] == 9 and m[1, 4] == 10 and m[2, 4] == 12 and m[3, 4] == 12
    assert m[4, 4] == 1 and m[2, 0] == 5 and m[3, 1] == 8


def test_beamset_packed_upload_matches_per_field():
    """BeamSet packs host beam fields into one buffer (one copy): every view
    equals the per-field conversion, scalars broadcast, wrong sizes raise."""
    import torch
    from temgymcore_gb300.gaussian import BeamSet, _f64
    from temgymcore_gb300.workloads import beamlet_field, gaussian_rays
    w = beamlet_field(seed=2, n_beams=37, det_shape=(8, 8), astigmatic=True)
    r = gaussian_rays(w["rays"])
    cpu = torch.device("cpu")
    b = BeamSet(r, cpu)
    n = 37
    for name, v, width in (("x", r.x, None), ("y", r.y, None), ("dx", r.dx, None), ("dy", r.dy, None),
                           ("pl", r.pathlength, None), ("wl", r.wavelength, None), ("theta", r.theta, None),
                           ("waist", r.waist_xy, 2), ("radii", r.radii_of_curv, 2)):
        got = getattr(b, name)
        assert got.is_contiguous()
        assert torch.equal(got, _f64(v, n, cpu, width)), name
    # a per-beam tensor field takes the per-field path with the same values
    r2 = r.derive(theta=torch.as_tensor(np.asarray(r.theta, np.float64)))
    b2 = BeamSet(r2, cpu)
    assert all(torch.equal(getattr(b, k), getattr(b2, k)) for k in ("x", "waist", "radii", "theta", "wl"))
    import pytest
    with pytest.raises((ValueError, AssertionError)):
        BeamSet(r.derive(theta=np.zeros(5)), cpu)


def test_coordinate_tuples():
    """tests/test_coordinates.py:7-41: PixelYX.to_pixels keeps the kind of
    its values, CoordXY.to_coords gives length-1 float arrays."""
    import temgymcore_gb300 as t
    for v, kind in ((17, "i"), (17.0, "f")):
        px = t.PixelYX(x=v, y=v + 6)
        pxs = px.to_pixels()
        assert isinstance(pxs, t.PixelsYX) and len(pxs.x) == 1 and len(pxs.y) == 1
        assert pxs.x[0] == px.x and pxs.y[0] == px.y
        assert pxs.x.dtype.kind == kind and pxs.y.dtype.kind == kind
    c = t.CoordXY(x=17.0, y=23.0).to_coords()
    assert isinstance(c, t.CoordsXY) and len(c.x) == 1 and c.x[0] == 17.0 and c.y[0] == 23.0
    assert c.x.dtype.kind == "f" and c.y.dtype.kind == "f"


def test_ray_to_vector_and_scan_grid_rotation():
    """tests/test_rays.py:106-115 (to_vector gives arrays) and
    tests/test_component.py:355-378 (one scan-grid column step is the pixel
    size rotated by the grid rotation, y axis flipped)."""
    import dataclasses
    import temgymcore_gb300 as t
    v = t.Ray(x=1.0, y=2.0, dx=0.1, dy=0.2, z=3.0, pathlength=4.0).to_vector()
    for f in dataclasses.fields(v):
        assert np.ndim(getattr(v, f.name)) == 1
    rng = np.random.default_rng(11)
    for rot in rng.uniform(-180.0, 180.0, 5):
        g = t.ScanGrid(z=0.0, rotation=float(rot), pixel_size=(0.1, 0.1), shape=(11, 11))
        mx0, my0 = g.pixels_to_metres((5, 5))
        mx1, my1 = g.pixels_to_metres((5, 6))
        th = np.deg2rad(rot)
        np.testing.assert_allclose([mx1 - mx0, my1 - my0], [np.cos(th) * 0.1, -np.sin(th) * 0.1], atol=1e-12)


def test_make_aperture_types():
    """utils.py:285-294: NumPy grids give a NumPy mask; torch grids a torch mask."""
    import torch
    from temgymcore_gb300.utils import make_aperture
    Y, X = np.meshgrid(np.linspace(-1, 1, 11), np.linspace(-1, 1, 11), indexing="ij")
    m = make_aperture(X, Y, aperture_ratio=0.4)
    assert isinstance(m, np.ndarray) and m.dtype == bool and m[5, 5] and not m[0, 0]
    assert np.array_equal(m, X ** 2 + Y ** 2 < (0.4 * np.max(np.abs(X))) ** 2)
    mt = make_aperture(torch.as_tensor(X), torch.as_tensor(Y), aperture_ratio=0.4)
    assert isinstance(mt, torch.Tensor) and np.array_equal(mt.numpy(), m)


def test_small_reference_helpers():
    """multi_cumsum_inplace (utils.py:47-80), FresnelPropagator
    (utils.py:245-262, NumPy and torch agree with the oracle's restatement),
    the 2x2 matrix helpers (gaussian.py:180-222), isnamedtuple."""
    import torch
    import temgymcore_gb300 as t
    from oracle import field as OF
    from temgymcore_gb300 import gaussian as G
    from temgymcore_gb300.tree_utils import isnamedtuple
    from temgymcore_gb300.utils import FresnelPropagator, fresnel_lens_imaging_solution, multi_cumsum_inplace
    v = np.ones(10)
    multi_cumsum_inplace(v, np.array([3, 2, 3]), 0.0)
    # restart one index after each boundary: [0,1,2,3] [0,1,2] [0,1,...]
    np.testing.assert_array_equal(v, [0, 1, 2, 3, 0, 1, 2, 0, 1, 2])
    rng = np.random.default_rng(0)
    u = rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))
    ref = OF.fresnel_tf(u, 1e-3, 5e-7, 0.01)
    np.testing.assert_allclose(FresnelPropagator(u, 1e-3, 5e-7, 0.01), ref, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(FresnelPropagator(torch.as_tensor(u), 1e-3, 5e-7, 0.01).numpy(), ref,
                               rtol=1e-12, atol=1e-12)
    Y, X = np.meshgrid(np.arange(16) * 1e-5, np.arange(16) * 1e-5, indexing="ij")
    np.testing.assert_allclose(fresnel_lens_imaging_solution(u, Y, X, 1e-5, 5e-7, 0.01, 0.02, 0.03),
                               OF.fresnel_thin_lens(u, X, Y, 1e-5, 5e-7, 0.01, 0.02, 0.03), rtol=1e-12, atol=1e-12)
    M, N2, v2 = rng.normal(size=(2, 2)), rng.normal(size=(2, 2)), rng.normal(size=2)
    np.testing.assert_allclose(G.matrix_vector_mul(M, v2), M @ v2)
    np.testing.assert_allclose(G.matrix_matrix_mul(M, N2), M @ N2)
    np.testing.assert_allclose(G.matrix_quadratic_mul(v2, M), v2 @ M @ v2)
    w = rng.normal(size=(5, 2))
    np.testing.assert_allclose(G.matrix_linear_mul(v2, M, w), w @ (M.T @ v2))
    B = rng.normal(size=(3, 2, 2))
    np.testing.assert_allclose(G.matrix_matrix_matrix_mul(B, B, B), B @ B @ np.swapaxes(B, 1, 2))
    assert isnamedtuple(t.DescanError()) and not isnamedtuple((1, 2))
