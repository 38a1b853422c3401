"""tg_trace_image: the per-SM shared-memory histogram path gives the same
histogram as the global-atomic path (tg_trace_fwd) and as a host bincount of
the kernel's own pixel indices, bit for bit: spread and single-pixel hit
patterns (the latter drives each uint16 counter to its per-flush maximum),
odd pixel counts, the unaligned (one ray per thread) variant, and
accumulation into int32 and int64 histograms that already hold counts."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup(n, shape, spread, offset=0, seed=0):
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda", 0)

    def col(v):  # optionally misaligned by `offset` elements (disables the float4 path)
        t = torch.empty(n + offset, dtype=torch.float32, device=dev)
        t[offset:] = torch.from_numpy(v.astype(np.float32)).to(dev)
        return t[offset:]
    x, y = (col(rng.uniform(-1e-3, 1e-3, n) * spread) for _ in range(2))
    dx, dy = (col(rng.normal(0, 1e-3, n) * spread) for _ in range(2))
    model = build_model([{"kind": "lens", "z": 0.5, "focal_length": 0.2},
                         {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": shape}])
    m, keep = pack_model(model)
    rin = _rays_struct(n, x, y, dx, dy, None, 0.0, None, 0.0)
    o = [torch.empty(n, device=dev) for _ in range(4)]
    rout = _rays_struct(n, *o, None, 0.0, None, 0.0)
    # the structs hold raw pointers: the tensors must outlive the calls
    return m, (keep, x, y, dx, dy, o), rin, rout, model[-1]._tg_grid(), dev


def _run(n, shape, spread, dtype=torch.int64, offset=0, prefill=0):
    from temgymcore_gb300 import _native as N
    lib = N.lib()
    m, keep, rin, rout, g, dev = _setup(n, shape, spread, offset)
    h, w = shape
    i64 = 1 if dtype == torch.int64 else 0
    ws_bytes = lib.tg_trace_image_workspace(n, C.byref(g))
    assert ws_bytes > 0  # the shared-memory path is taken
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    py, px = (torch.empty(n, dtype=torch.int32, device=dev) for _ in range(2))
    h_sh = torch.full((h, w), prefill, dtype=dtype, device=dev)
    N.check(lib.tg_trace_image(C.byref(m), C.byref(rin), C.byref(rout), None, C.byref(g), N.ptr(py),
                               N.ptr(px), N.ptr(h_sh), i64, N.ptr(ws), ws_bytes, N.stream_ptr()),
            "tg_trace_image")
    h_gl = torch.full((h, w), prefill, dtype=dtype, device=dev)
    N.check(lib.tg_trace_fwd(C.byref(m), C.byref(rin), C.byref(rout), None, C.byref(g), None, None,
                             N.ptr(h_gl), i64, N.stream_ptr()), "tg_trace_fwd")
    torch.cuda.synchronize()
    pyh, pxh = py.cpu().numpy(), px.cpu().numpy()
    ok = (pyh >= 0) & (pyh < h) & (pxh >= 0) & (pxh < w)
    ref = np.bincount((pyh[ok].astype(np.int64) * w + pxh[ok]), minlength=h * w).reshape(h, w) + prefill
    del keep
    return h_sh.cpu().numpy(), h_gl.cpu().numpy(), ref


@pytest.mark.parametrize("shape", [(64, 64), (63, 65), (320, 320)])
def test_trace_image_spread(cuda, shape):
    # 320 x 320 = 102,400 pixels: the largest detector of the shared path (200 KB)
    n = max((1 << 22) + 3, 33 * shape[0] * shape[1])
    h_sh, h_gl, ref = _run(n, shape, spread=0.08 * shape[0] / 64)
    assert np.array_equal(h_sh, ref) and np.array_equal(h_gl, ref)
    assert ref.sum() > n // 2


def test_trace_image_one_pixel_many_carries(cuda):
    # every ray in the centre pixel: 10M rays over the SMs, about 66k hits per
    # CTA on one uint16 counter, which moves 16384 counts into the histogram
    # each time it reaches that value
    n = 10_000_000
    h_sh, h_gl, ref = _run(n, (32, 32), spread=0.0)
    assert np.array_equal(h_sh, ref) and np.array_equal(h_gl, ref)
    assert int(ref.max()) == n


@pytest.mark.parametrize("shape", [(64, 64), (300, 300)])
def test_trace_image_aligned_int32_prefilled(cuda, shape):
    # the four-rays-per-thread kernels with an int32 histogram (the
    # prefetching shared-memory variant at 64 x 64; 300 x 300 leaves no room
    # for the prefetch slots), counts added to a prefilled histogram
    n = (1 << 22) + 5
    h_sh, h_gl, ref = _run(n, shape, spread=0.08 * shape[0] / 64, dtype=torch.int32, prefill=3)
    assert np.array_equal(h_sh, ref) and np.array_equal(h_gl, ref)


@pytest.mark.parametrize("dtype", [torch.int32, torch.int64])
def test_trace_image_unaligned_and_prefilled(cuda, dtype):
    n = (1 << 21) + 1
    h_sh, h_gl, ref = _run(n, (48, 40), spread=0.05, dtype=dtype, offset=1, prefill=7)
    assert np.array_equal(h_sh, ref) and np.array_equal(h_gl, ref)


def test_trace_image_workspace_policy(cuda):
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.components import Detector
    lib = N.lib()
    g_small = Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(256, 256))._tg_grid()
    g_big = Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(512, 512))._tg_grid()
    assert lib.tg_trace_image_workspace(1 << 24, C.byref(g_small)) > 0
    assert lib.tg_trace_image_workspace(65536, C.byref(g_small)) == 0   # few rays per pixel
    assert lib.tg_trace_image_workspace(1 << 26, C.byref(g_big)) == 0   # detector above the shared budget


@pytest.mark.parametrize("idt", [torch.int32, torch.int64])
def test_into_image_pixel_indices(cuda, idt):
    """Detector.into_image given (py, px): tg_hist_pixels (shared-memory path
    at this size, global atomics below it) equals a host bincount; indices
    outside the detector, including beyond int32 for int64 input, are dropped."""
    import temgymcore_gb300 as t
    rng = np.random.default_rng(3)
    det = t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(40, 56))
    for n in (1 << 21, 5000):
        py = rng.integers(-3, 44, n)
        px = rng.integers(-5, 60, n)
        if idt == torch.int64:
            py[::97] = 2 ** 33 + 5   # would wrap into range if narrowed to int32
            px[::89] = -(2 ** 40)
        acc = torch.full((40, 56), 2, dtype=torch.int64, device=cuda)
        out = det.into_image((torch.tensor(py, dtype=idt), torch.tensor(px, dtype=idt)), acc)
        ok = (py >= 0) & (py < 40) & (px >= 0) & (px < 56)
        ref = np.bincount(py[ok] * 56 + px[ok], minlength=40 * 56).reshape(40, 56) + 2
        assert np.array_equal(out.cpu().numpy(), ref), n


@pytest.mark.parametrize("hdt", [torch.int32, torch.int64])
def test_hist_pixels_carry_on_one_word(cuda, hdt):
    """Every hit on the two pixels that share one packed shared-memory word:
    each CTA drives both uint16 halves past 16384 four times (the carry
    into the histogram must leave the neighbouring half intact), on top of
    prefilled counts; the remaining hits stay in the per-CTA rows."""
    import temgymcore_gb300 as t
    n = 24_000_001
    rng = np.random.default_rng(9)
    det = t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(30, 30))
    b = rng.integers(0, 2, n)  # bins 2 * 225 + b: one packed word
    py = torch.tensor(np.full(n, 15, np.int32), device=cuda)
    px = torch.tensor((b + 0).astype(np.int32), device=cuda)
    acc = torch.full((30, 30), 5, dtype=hdt, device=cuda)
    out = det.into_image((py, px), acc)
    ref = np.full((30, 30), 5, np.int64)
    ref[15, 0] += int((b == 0).sum())
    ref[15, 1] += int((b == 1).sum())
    assert np.array_equal(out.cpu().numpy().astype(np.int64), ref)


def test_into_image_rays_shared_vs_global(cuda):
    """Detector.into_image given rays (tg_bin_image, shared-memory path) equals
    tg_bin (global atomics) and the oracle's binning of the same coordinates."""
    import oracle
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    rng = np.random.default_rng(4)
    n = (1 << 21) + 7
    det = t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(48, 48))
    x = torch.tensor(rng.normal(0, 1.5e-4, n).astype(np.float32), device=cuda)
    y = torch.tensor(rng.normal(0, 1.5e-4, n).astype(np.float32), device=cuda)
    assert N.lib().tg_hist_workspace(n, 48, 48) > 0
    img = det.into_image(t.Ray(x=x, y=y, dx=0.0, dy=0.0, z=0.0, pathlength=0.0))
    g = det._tg_grid()
    ref_gl = torch.zeros((48, 48), dtype=torch.int64, device=cuda)
    N.check(N.lib().tg_bin(n, N.ptr(x), N.ptr(y), None, C.byref(g), None, None, N.ptr(ref_gl), 1,
                           N.stream_ptr()), "tg_bin")
    assert torch.equal(img, ref_gl)
    gd = {"pixel_size": (1e-5, 1e-5), "shape": (48, 48)}
    py, px = oracle.metres_to_pixels(gd, x.cpu().numpy().astype(np.float64), y.cpu().numpy().astype(np.float64))
    assert np.array_equal(img.cpu().numpy(), oracle.into_image(gd, py, px))


def test_trace_plan_shared_hist_graph(cuda):
    """TracePlan on the shared-memory histogram path (workspace held by the
    plan) equals trace_to_image, and replays inside a CUDA graph."""
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    rng = np.random.default_rng(8)
    n = 1 << 22
    model = [t.Lens(z=0.5, focal_length=0.2),
             t.Detector(z=1.0, pixel_size=(1e-5, 1e-5), shape=(64, 64))]
    xs = [torch.tensor((rng.uniform(-1, 1, n) * s).astype(np.float32), device=cuda)
          for s in (8e-5, 8e-5, 8e-5, 8e-5)]
    assert N.lib().tg_trace_image_workspace(n, C.byref(model[-1]._tg_grid())) > 0
    out, pix, img = t.trace_to_image(t.Ray(x=xs[0], y=xs[1], dx=xs[2], dy=xs[3], z=0.0, pathlength=0.0),
                                     model)
    assert int(img.sum()) > n // 2
    plan = t.TracePlan(model, *xs, detector=model[-1], pixels=True)
    plan.run()
    assert torch.equal(plan.image, img) and torch.equal(plan.pix[0], pix.y)
    g = plan.capture()
    plan.image.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(plan.image, 2 * img)


@pytest.mark.parametrize("n", [2047, 2048, 4099, 2 * 152 * 2048 + 1234])
def test_vector_and_scalar_variants_agree_bit_for_bit(cuda, n):
    """Aligned arrays take the four-rays-per-thread kernels (16-byte vector
    loads and stores); a one-element offset view of the same data takes the
    one-ray-per-thread kernels.  The chain's arithmetic is written with
    explicit fused multiply-adds, so both give every output (coordinates,
    float64 pathlength, z, amplitude, pixel indices, global and shared-memory
    histograms) bit for bit: through a lens, an aperture and a biprism, with
    per-ray z and pathlength inputs, at ragged and whole sizes."""
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import build_model
    lib = N.lib()
    rng = np.random.default_rng(n)
    shape = (64, 64)
    model = build_model([{"kind": "lens", "z": 0.5, "focal_length": 0.2},
                         {"kind": "aperture", "z": 0.6, "radius": 2.5e-4},
                         {"kind": "biprism", "z": 0.7, "def_x": 3e-5},
                         {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": shape}])
    m, keep_m = pack_model(model)
    g = model[-1]._tg_grid()
    cols = {"x": rng.uniform(-4e-4, 4e-4, n), "y": rng.uniform(-4e-4, 4e-4, n),
            "dx": rng.normal(0, 5e-4, n), "dy": rng.normal(0, 5e-4, n)}
    z = rng.uniform(-1e-3, 1e-3, n)
    pl = rng.uniform(0, 1e-2, n)
    amp = rng.uniform(0.5, 1.0, n)

    def put(v, dt, off):
        t = torch.empty(n + off, dtype=dt, device=cuda)
        t[off:] = torch.from_numpy(np.asarray(v)).to(dt).to(cuda)
        return t[off:]

    def run(off, shared):
        xs = [put(cols[k], torch.float32, off) for k in ("x", "y", "dx", "dy")]
        zt, plt, at = put(z, torch.float64, off), put(pl, torch.float64, off), put(amp, torch.float32, off)
        rin = _rays_struct(n, *xs, zt, 0.0, plt, 0.0, at)
        o = [put(np.zeros(n), torch.float32, off) for _ in range(4)]
        opl, oz, oa = put(np.zeros(n), torch.float64, off), put(np.zeros(n), torch.float64, off), \
            put(np.zeros(n), torch.float32, off)
        rout = _rays_struct(n, *o, oz, 0.0, opl, 0.0, oa)
        py, px = put(np.zeros(n), torch.int32, off), put(np.zeros(n), torch.int32, off)
        hist = torch.zeros(shape, dtype=torch.int64, device=cuda)
        if shared:
            ws_bytes = lib.tg_trace_image_workspace(n, C.byref(g))
            assert ws_bytes > 0
            ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
            N.check(lib.tg_trace_image(C.byref(m), C.byref(rin), C.byref(rout), None, C.byref(g),
                                       N.ptr(py), N.ptr(px), N.ptr(hist), 1, N.ptr(ws), ws_bytes,
                                       N.stream_ptr()), "tg_trace_image")
        else:
            N.check(lib.tg_trace_fwd(C.byref(m), C.byref(rin), C.byref(rout), None, C.byref(g),
                                     N.ptr(py), N.ptr(px), N.ptr(hist), 1, N.stream_ptr()), "tg_trace_fwd")
        torch.cuda.synchronize()
        return [t.cpu().numpy() for t in (*o, opl, oz, oa, py, px, hist)]

    modes = [False] + ([True] if n >= 32 * shape[0] * shape[1] else [])
    for shared in modes:
        a, b = run(0, shared), run(1, shared)
        for u, v in zip(a, b):
            assert np.array_equal(u, v), shared
        assert a[-1].sum() > 0
    assert N.error_word() == 0
