"""GPU parity of the fused ray chain, binning, histogram and adjoint against
the float64 oracle.  Tolerances: coordinates <= 1e-6 normwise relative
(float32 ray state); pixel indices and histograms bit-exact given the same
float32 coordinates; gradients <= 1e-4 normwise relative."""
import numpy as np
import pytest
import torch

import oracle
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu

COORD_TOL = 1e-6


def T():
    import temgymcore_gb300 as t
    return t


def np_(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def _grid(spec):
    return {k: spec[k] for k in ("pixel_size", "shape", "rotation", "centre", "flip_y") if k in spec}


def _cmp_trace(out, ref, tol=COORD_TOL):
    for k in ("x", "y", "dx", "dy"):
        e = normwise_err(np_(getattr(out, k)), getattr(ref, k))
        assert e <= tol, (k, e)
    e = normwise_err(np_(out.pathlength), ref.pathlength)
    assert e <= 1e-9, ("pathlength", e)


def _run(w, cuda):
    t = T()
    from temgymcore_gb300.workloads import build_model
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                z=w["z"], pathlength=w["pathlength"])
    return ray, build_model(w["model"])


def test_readme_quickstart_gpu(kats, cuda):
    t = T()
    from temgymcore_gb300.workloads import build_model
    q = kats["readme_quickstart"]
    out = t.run_to_end(t.Ray(**q["ray"]), build_model(q["model"]))
    for k, v in q["expected"].items():
        assert abs(float(np_(getattr(out, k))) - v) <= 1e-6 * max(1.0, abs(v)), k


def test_plain_trace_parity_and_bit_exact_binning(cuda):
    t = T()
    from temgymcore_gb300.workloads import plain_trace
    w = plain_trace(seed=0, n=65536)
    ray, model = _run(w, cuda)
    out, pix, img = t.trace_to_image(ray, model)
    ref = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], 0.0, 0.0), w["model"])
    _cmp_trace(out, ref)
    g = _grid(w["model"][-1])
    py, px = oracle.metres_to_pixels(g, np_(out.x).astype(np.float64), np_(out.y).astype(np.float64))
    assert np.array_equal(np_(pix.y), py) and np.array_equal(np_(pix.x), px)
    acc = oracle.into_image(g, py, px)
    assert img.dtype == torch.int64 and np.array_equal(np_(img), acc)
    assert int(np_(img).sum()) > 40000  # ~70% of the rays land on the 256x256 detector
    # the unfused API path gives the same answers
    out2 = t.run_to_end(ray, model)
    assert torch.equal(out2.x, out.x) and torch.equal(out2.pathlength, out.pathlength)
    det = model[-1]
    p2 = det.metres_to_pixels((out2.x, out2.y))
    assert torch.equal(p2.y, pix.y) and torch.equal(p2.x, pix.x)
    img2 = det.into_image(out2)
    assert torch.equal(img2, img)
    img3 = det.into_image(out2, torch.zeros((256, 256), dtype=torch.int32, device=cuda))
    assert np.array_equal(np_(img3), acc)
    assert t._native.error_word() == 0


def test_binning_adversarial_ties(cuda):
    """Coordinates on and next to pixel-rounding ties decide via float64."""
    t = T()
    det = t.Detector(z=0.0, pixel_size=(1e-5, 1e-5), shape=(256, 256))
    rng = np.random.default_rng(11)
    j = rng.integers(-140, 140, 20000)
    base = (j * 1e-5).astype(np.float32)  # exactly at (or within an ulp of) a tie
    nudge = rng.integers(-3, 4, j.size).astype(np.float32)
    x = np.nextafter(base, np.float32(np.inf) * np.sign(nudge)).astype(np.float32)
    x = np.where(nudge == 0, base, x)
    y = np.roll(x, 7)
    xt = torch.tensor(x, device=cuda)
    yt = torch.tensor(y, device=cuda)
    p = det.metres_to_pixels((xt, yt))
    g = {"pixel_size": (1e-5, 1e-5), "shape": (256, 256)}
    py, px = oracle.metres_to_pixels(g, x.astype(np.float64), y.astype(np.float64))
    assert np.array_equal(np_(p.y), py) and np.array_equal(np_(p.x), px)
    # rotated / off-centre / flipped grid
    det2 = t.Detector(z=0.0, pixel_size=(2e-5, 1e-5), shape=(100, 300), rotation=33.0,
                      centre=(1e-4, -3e-4), flip_y=True)
    g2 = {"pixel_size": (2e-5, 1e-5), "shape": (100, 300), "rotation": 33.0,
          "centre": (1e-4, -3e-4), "flip_y": True}
    p = det2.metres_to_pixels((xt, yt))
    py, px = oracle.metres_to_pixels(g2, x.astype(np.float64), y.astype(np.float64))
    assert np.array_equal(np_(p.y), py) and np.array_equal(np_(p.x), px)
    img = det2.into_image(t.Ray(x=xt, y=yt, dx=0.0, dy=0.0, z=0.0, pathlength=0.0))
    assert np.array_equal(np_(img), oracle.into_image(g2, py, px))


def test_nonfinite_and_saturating_pixels(cuda):
    t = T()
    det = t.Detector(z=0.0, pixel_size=(1e-5, 1e-5), shape=(16, 16))
    x = np.array([np.nan, np.inf, -np.inf, 1e30, -1e30, 3e4, 0.0, 5e-5], dtype=np.float32)
    y = np.array([0.0, 0.0, 1.0, 0.0, 0.0, -3e4, np.nan, 5e-5], dtype=np.float32)
    p = det.metres_to_pixels((torch.tensor(x, device=cuda), torch.tensor(y, device=cuda)))
    g = {"pixel_size": (1e-5, 1e-5), "shape": (16, 16)}
    py, px = oracle.metres_to_pixels(g, x.astype(np.float64), y.astype(np.float64))
    assert np.array_equal(np_(p.y), py) and np.array_equal(np_(p.x), px)
    assert t._native.error_word() & t._native.EW_NONFINITE
    assert t._native.error_word() == 0  # cleared by the previous read


@pytest.mark.parametrize("n", [0, 1, 3, 5, 4097])
def test_ragged_sizes_and_unaligned_views(n, cuda):
    t = T()
    rng = np.random.default_rng(n)
    buf = rng.normal(0, 1e-3, (4, n + 1)).astype(np.float32)
    tb = torch.tensor(buf, device=cuda)
    ray = t.Ray(x=tb[0, 1:], y=tb[1, 1:], dx=tb[2, 1:], dy=tb[3, 1:], z=0.0, pathlength=0.25)
    spec = [{"kind": "lens", "z": 0.3, "focal_length": 0.1},
            {"kind": "deflector", "z": 0.4, "def_x": 1e-4, "def_y": 0.0},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (64, 64)}]
    from temgymcore_gb300.workloads import build_model
    out, pix, img = t.trace_to_image(ray, build_model(spec))
    ref = oracle.run_to_end(ORay.from_f32(buf[0, 1:], buf[1, 1:], buf[2, 1:], buf[3, 1:], 0.0, 0.25), spec)
    if n:
        _cmp_trace(out, ref)
        py, px = oracle.metres_to_pixels(_grid(spec[-1]), np_(out.x).astype(np.float64),
                                         np_(out.y).astype(np.float64))
        assert np.array_equal(np_(pix.y), py) and np.array_equal(np_(pix.x), px)
        assert np.array_equal(np_(img), oracle.into_image(_grid(spec[-1]), py, px))
    else:
        assert out.x.numel() == 0 and int(img.sum()) == 0


def _full_chain_spec():
    rng = np.random.default_rng(5)
    err = dict(zip(["pxo_pxi", "pxo_pyi", "pyo_pxi", "pyo_pyi", "sxo_pxi", "sxo_pyi", "syo_pxi",
                    "syo_pyi", "offpxi", "offpyi", "offsxi", "offsyi"],
                   rng.normal(0, 1e-2, 12).tolist()))
    return [{"kind": "source", "z": 0.0},
            {"kind": "lens", "z": 0.1, "focal_length": 0.05},
            {"kind": "scanner", "z": 0.15, "scan_pos_x": 1e-5, "scan_pos_y": -2e-5,
             "scan_tilt_x": 1e-4, "scan_tilt_y": -1e-4},
            {"kind": "descanner", "z": 0.15, "scan_pos_x": 1e-5, "scan_pos_y": -2e-5,
             "scan_tilt_x": 1e-4, "scan_tilt_y": -1e-4, "descan_error": err},
            {"kind": "deflector", "z": 0.2, "def_x": 2e-4, "def_y": -1e-4},
            {"kind": "rotator", "z": 0.25, "angle": 23.0},
            {"kind": "biprism", "z": 0.3, "def_x": 5e-4},
            {"kind": "thicklens", "z_po": 0.4, "z_pi": 0.41, "focal_length": 0.2},
            {"kind": "plane", "z": 0.5},
            {"kind": "detector", "z": 0.8, "pixel_size": (2e-5, 2e-5), "shape": (128, 128)}]


def test_full_component_chain_per_ray_z_and_pathlength(cuda):
    t = T()
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(9)
    n = 10001
    x, y, dx, dy = (rng.normal(0, 1e-4, n).astype(np.float32) for _ in range(4))
    z = rng.uniform(-0.01, 0.0, n)
    pl = rng.uniform(0.0, 1.0, n)
    spec = _full_chain_spec()
    ray = t.Ray(x=torch.tensor(x, device=cuda), y=torch.tensor(y, device=cuda),
                dx=torch.tensor(dx, device=cuda), dy=torch.tensor(dy, device=cuda),
                z=torch.tensor(z, device=cuda), pathlength=torch.tensor(pl, device=cuda))
    out = t.run_to_end(ray, build_model(spec))
    ref = oracle.run_to_end(ORay.from_f32(x, y, dx, dy, z, pl), spec)
    # ten components incl. a 5 cm lens: float32 state rounded exactly after
    # every component already differs from float64 by 1.1e-6 (dx) here
    _cmp_trace(out, ref, tol=2e-6)
    assert abs(out.z - float(np.mean(ref.z))) < 1e-12


def test_aperture_blocks_histogram(cuda):
    t = T()
    rng = np.random.default_rng(1)
    n = 20000
    x = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    y = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    spec = [{"kind": "aperture", "z": 0.1, "radius": 6e-4, "centre": (1e-4, 0.0)},
            {"kind": "detector", "z": 0.2, "pixel_size": (1e-5, 1e-5), "shape": (256, 256)}]
    from temgymcore_gb300.workloads import build_model
    ray = t.Ray(x=torch.tensor(x, device=cuda), y=torch.tensor(y, device=cuda), dx=0.0, dy=0.0,
                z=0.0, pathlength=0.0)
    out, pix, img = t.trace_to_image(ray, build_model(spec))
    ref = oracle.run_to_end(ORay.from_f32(x, y, np.zeros(n), np.zeros(n), 0.0, 0.0), spec)
    g = _grid(spec[-1])
    py, px = oracle.metres_to_pixels(g, np_(out.x).astype(np.float64), np_(out.y).astype(np.float64))
    assert np.array_equal(np_(img), oracle.into_image(g, py, px, mask=ref.alive))
    assert int(np_(img).sum()) == int(ref.alive.sum()) < n


# ------------------------------------------------------------------ adjoint

def _cs_outputs(w, spec, which, h=1e-30):
    """Complex-step derivatives of all outputs w.r.t. a ray field or param."""
    kind, key = which
    f64 = lambda a: np.asarray(a, np.float32).astype(np.complex128)  # noqa: E731
    x, y, dx, dy = f64(w["x"]), f64(w["y"]), f64(w["dx"]), f64(w["dy"])
    spec = [dict(c) for c in spec]
    if kind == "ray":
        d = {"x": x, "y": y, "dx": dx, "dy": dy}
        d[key] = d[key] + 1j * h
        x, y, dx, dy = d["x"], d["y"], d["dx"], d["dy"]
    else:
        i, name = key
        if name.startswith("descan_error."):
            e = dict(spec[i]["descan_error"])
            e[name.split(".")[1]] = e.get(name.split(".")[1], 0.0) + 1j * h
            spec[i]["descan_error"] = e
        else:
            spec[i][name] = spec[i][name] + 1j * h
    o = oracle.run_to_end(ORay(x, y, dx, dy, np.complex128(w.get("z", 0.0)),
                               np.complex128(w.get("pathlength", 0.0))), spec)
    return [np.imag(getattr(o, k)) / h for k in ("x", "y", "dx", "dy", "pathlength")]


def test_adjoint_matches_complex_step(cuda):
    t = T()
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(21)
    n = 4099
    w = {"x": rng.normal(0, 1e-4, n).astype(np.float32), "y": rng.normal(0, 1e-4, n).astype(np.float32),
         "dx": rng.normal(0, 1e-3, n).astype(np.float32), "dy": rng.normal(0, 1e-3, n).astype(np.float32),
         "z": 0.0, "pathlength": 0.0}
    spec = _full_chain_spec()
    comps = build_model(spec)
    # make parameters differentiable
    import dataclasses
    pnames = [(1, "focal_length"), (1, "z"), (2, "scan_pos_x"), (2, "scan_tilt_y"), (3, "scan_pos_y"),
              (3, "descan_error.pxo_pxi"), (3, "descan_error.offsyi"), (4, "def_x"), (4, "def_y"),
              (5, "angle"), (6, "def_x"), (7, "focal_length"), (7, "z_pi"), (9, "z")]
    tens = {}
    for (i, name) in pnames:
        c = comps[i]
        if name.startswith("descan_error."):
            dn = name.split(".")[1]
            v = torch.tensor(float(getattr(c.descan_error, dn)), dtype=torch.float64, requires_grad=True)
            comps[i] = dataclasses.replace(c, descan_error=c.descan_error._replace(**{dn: v}))
        else:
            v = torch.tensor(float(getattr(c, name)), dtype=torch.float64, requires_grad=True)
            comps[i] = dataclasses.replace(c, **{name: v})
        tens[(i, name)] = v
    xs = {k: torch.tensor(w[k], device=cuda, requires_grad=True) for k in ("x", "y", "dx", "dy")}
    ray = t.Ray(x=xs["x"], y=xs["y"], dx=xs["dx"], dy=xs["dy"], z=0.0, pathlength=0.0)
    out = t.run_to_end(ray, comps)
    g = [rng.normal(0, 1, n).astype(np.float32) for _ in range(4)]
    gpl = rng.normal(0, 1, n)
    loss = sum((torch.tensor(gi, device=cuda) * o.double().float()).double().sum()
               for gi, o in zip(g, (out.x, out.y, out.dx, out.dy)))
    loss = loss + (torch.tensor(gpl, device=cuda) * out.pathlength).sum()
    loss.backward()
    gv = [gi.astype(np.float64) for gi in g] + [gpl]
    for k in ("x", "y", "dx", "dy"):
        d = _cs_outputs(w, spec, ("ray", k))
        ref = sum(gi * di for gi, di in zip(gv, d))
        e = normwise_err(np_(xs[k].grad), ref)
        assert e < 1e-4, (k, e)
    for key, v in tens.items():
        d = _cs_outputs(w, spec, ("param", key))
        ref = float(sum((gi * di).sum() for gi, di in zip(gv, d)))
        got = float(v.grad)
        assert abs(got - ref) <= 1e-4 * max(abs(ref), 1e-12) + 1e-3 * _scale(gv, d), (key, got, ref)


def _scale(gv, d):
    return float(sum((np.abs(gi * di)).sum() for gi, di in zip(gv, d))) * 1e-3


def test_readme_gradients_gpu(kats, cuda):
    t = T()
    q = kats["readme_quickstart"]
    f = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    zl = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    det = t.Detector(z=1.0, pixel_size=(0.01, 0.01), shape=(128, 128))
    out = t.run_to_end(t.Ray(**q["ray"]), [t.Lens(z=zl, focal_length=f), det])
    out.x.backward()
    np.testing.assert_allclose([float(f.grad), float(zl.grad)], kats["readme_grads"]["dx_out_d_f_and_z"],
                               rtol=1e-6)
    x = torch.tensor(0.01, device=cuda, requires_grad=True)
    out = t.run_to_end(t.Ray(x=x, y=0.2, dx=0.3, dy=0.4, z=0.0, pathlength=0.6),
                       [t.Lens(z=0.5, focal_length=1.0), det])
    out.dx.backward()
    assert abs(float(x.grad) - kats["readme_grads"]["ddx_out_dx_in"]) < 1e-6


def test_trace_plan_and_graph_match_api(cuda):
    t = T()
    from temgymcore_gb300.workloads import build_model, plain_trace
    w = plain_trace(seed=3, n=10000)
    model = build_model(w["model"])
    xs = [torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy")]
    out, pix, img = t.trace_to_image(t.Ray(x=xs[0], y=xs[1], dx=xs[2], dy=xs[3], z=0.0, pathlength=0.0),
                                     model)
    plan = t.TracePlan(model, *xs, detector=model[-1], pixels=True)
    plan.run()
    assert torch.equal(plan.out[0], out.x) and torch.equal(plan.pathlength, out.pathlength)
    assert torch.equal(plan.image, img) and torch.equal(plan.pix[1], pix.x)
    g = plan.capture()
    plan.image.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(plan.image, 2 * img)


def test_trace_adj_one_call_matches_composition(cuda):
    """tg_trace_adj (forward + residual + adjoint in one call) equals
    tg_trace_fwd, 2 (out - target) and tg_trace_vjp done separately."""
    import ctypes as C
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import build_model
    N.register("tg_trace_adj_workspace", C.c_size_t, [C.c_int64, C.POINTER(N.TgModel)])
    N.register("tg_trace_adj", C.c_int, [C.POINTER(N.TgModel), C.POINTER(N.TgRays), C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p])
    N.register("tg_get_last_error_word", C.c_uint32, [])
    t = T()
    rng = np.random.default_rng(4)
    n = 5003
    w = {k: torch.tensor(rng.normal(0, s, n).astype(np.float32), device=cuda)
         for k, s in (("x", 1e-4), ("y", 1e-4), ("dx", 1e-3), ("dy", 1e-3))}
    tx, ty = (torch.tensor(rng.normal(0, 1e-4, n).astype(np.float32), device=cuda) for _ in range(2))
    m, keep = pack_model(build_model(_full_chain_spec()))
    ns = 2 * m.n_components
    rin = _rays_struct(n, w["x"], w["y"], w["dx"], w["dy"], None, 0.0, None, 0.0)
    ws = torch.empty(N.lib().tg_trace_adj_workspace(n, C.byref(m)) + 256, dtype=torch.uint8, device=cuda)
    wp = ws.data_ptr() + (-ws.data_ptr()) % 256
    dpar = torch.full((ns, 4), 7.0, dtype=torch.float64, device=cuda)
    g = [torch.empty(n, device=cuda) for _ in range(4)]
    gin = _rays_struct(n, *g, None, 0.0, None, 0.0)
    N.check(N.lib().tg_trace_adj(C.byref(m), C.byref(rin), tx.data_ptr(), ty.data_ptr(), dpar.data_ptr(),
                                 C.byref(gin), wp, ws.numel() - 256, N.stream_ptr()))
    # composition
    o = [torch.empty(n, device=cuda) for _ in range(4)]
    rout = _rays_struct(n, *o, None, 0.0, None, 0.0)
    N.check(N.lib().tg_trace_fwd(C.byref(m), C.byref(rin), C.byref(rout), None, None, None, None, None, 0,
                                 N.stream_ptr()))
    gx, gy = 2 * (o[0] - tx), 2 * (o[1] - ty)
    z = torch.zeros(n, device=cuda)
    gout = _rays_struct(n, gx.contiguous(), gy.contiguous(), z, z, None, 0.0, None, 0.0)
    raw = torch.zeros((ns, 4), dtype=torch.float64, device=cuda)
    g2 = [torch.empty(n, device=cuda) for _ in range(4)]
    gin2 = _rays_struct(n, *g2, None, 0.0, None, 0.0)
    ws2 = torch.empty(max(8, N.lib().tg_trace_vjp_workspace(n, C.byref(m))), dtype=torch.uint8, device=cuda)
    N.check(N.lib().tg_trace_vjp(C.byref(m), C.byref(rin), C.byref(gout), C.byref(gin2), raw.data_ptr(),
                                 ws2.data_ptr(), ws2.numel(), N.stream_ptr()))
    torch.cuda.synchronize()
    assert normwise_err(np_(dpar), np_(raw)) < 1e-6
    for a, b in zip(g, g2):
        assert normwise_err(np_(a), np_(b)) < 1e-6
    assert N.lib().tg_get_last_error_word() == 0


@pytest.mark.parametrize("dircos", [False, True])
def test_lean_adjoint_matches_general(cuda, dircos):
    """Chains without biprisms, per-ray z or an upstream pathlength gradient
    take the lean adjoint (state and adjoint only, 8 rays a thread); the same
    call with a zero pathlength gradient array takes the general adjoint.
    Input gradients and per-step sums agree to float32 rounding, through
    lenses, scanners / descanners with descan error, a deflector, a rotator,
    an aperture and a thick lens, with paraxial and direction-cosine free
    space, over whole 8-ray groups and a ragged tail."""
    import ctypes as C
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.propagator import FreeSpaceDirCosine
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import build_model
    spec = [c for c in _full_chain_spec() if c["kind"] != "biprism"]
    spec.insert(5, {"kind": "aperture", "z": 0.27, "radius": 5e-4})
    m, keep = pack_model(build_model(spec), FreeSpaceDirCosine() if dircos else None)
    ns = 2 * m.n_components
    rng = np.random.default_rng(17)
    n = 3 * 152 * 2048 + 13
    w = [torch.tensor(rng.normal(0, s, n).astype(np.float32), device=cuda) for s in (1e-4, 1e-4, 1e-3, 1e-3)]
    g = [torch.tensor(rng.normal(0, 1, n).astype(np.float32), device=cuda) for _ in range(4)]
    rin = _rays_struct(n, *w, None, 0.0, None, 0.0)
    ws = torch.empty(N.lib().tg_trace_vjp_workspace(n, C.byref(m)), dtype=torch.uint8, device=cuda)
    zpl = torch.zeros(n, dtype=torch.float64, device=cuda)
    res = []
    for pl in (None, zpl):
        gout = _rays_struct(n, *g, None, 0.0, pl, 0.0)
        gi = [torch.empty(n, device=cuda) for _ in range(4)]
        gin = _rays_struct(n, *gi, None, 0.0, None, 0.0)
        raw = torch.zeros((ns, 4), dtype=torch.float64, device=cuda)
        N.check(N.lib().tg_trace_vjp(C.byref(m), C.byref(rin), C.byref(gout), C.byref(gin), raw.data_ptr(),
                                     ws.data_ptr(), ws.numel(), N.stream_ptr()), "tg_trace_vjp")
        torch.cuda.synchronize()
        res.append(([np_(t) for t in gi], np_(raw)))
    (gl, rl), (gg, rg) = res
    for a, b in zip(gl, gg):
        assert normwise_err(a, b) < 1e-6
    assert normwise_err(rl, rg) < 1e-6
    assert np.abs(rl).max() > 0 and N.error_word() == 0
