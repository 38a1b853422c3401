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


def test_trace_image_one_pixel_many_flushes(cuda):
    # every ray in the centre pixel: 10M rays over the SMs, several flushes per
    # CTA with 61,440 hits per counter between flushes
    n = 10_000_000
    h_sh, h_gl, ref = _run(n, (32, 32), spread=0.0)
    assert np.array_equal(h_sh, ref) and np.array_equal(h_gl, ref)
    assert int(ref.max()) == n


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
