"""tg_field_direct_noalloc: the direct beamlet-field sum for callers that
cannot allocate device memory (their allocator belongs to another framework,
or the device is pre-sized and allocation after start-up is not allowed).
The entry point keeps its scratch in a fixed array inside the library.

Called through the C ABI twice in a row; each result must match the regular
entry points (tg_field_prep + tg_field_eval, direct method) to the direct
kernel's tolerance and the float64 oracle on a pixel sample, and requests
beyond the stated limits are rejected.
This file sorts last so a failure here does not hide any other test."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-5  # normwise relative; the two paths only differ in beam chunking
SCRATCH = 32 << 20  # bytes of the library's fixed array


def _part(n):
    """Bytes ahead of the partial image in the array (the header's part(n))."""
    r = lambda v: (v + 255) // 256 * 256  # noqa: E731
    return r(r(r(96 * n) + 128 * n) + 256)


def _max_rows(n, w):
    return (SCRATCH - _part(n)) // (8 * w)


def _lib():
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300 import gaussian as G
    N.register("tg_field_direct_noalloc", C.c_int,
               [C.POINTER(N.TgModel), C.POINTER(G.TgBeams), C.POINTER(G.TgPixelMap), C.c_void_p,
                C.c_void_p])
    return N.lib()


def test_noalloc_matches_regular_direct_path(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.gaussian import BeamSet, pixel_map
    from temgymcore_gb300.run import pack_model
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    lib = _lib()
    w = beamlet_field(seed=3, n_beams=3000, det_shape=(96, 160), det_px=3e-5, astigmatic=True)
    rays, comps = gaussian_rays(w["rays"]), build_model(w["model"])
    ref = t.FieldPlan(rays, comps, method="direct").evaluate("direct").clone()
    beams = BeamSet(rays, cuda)
    pm = pixel_map(comps[-1])
    m, keep = pack_model(comps)
    outs = []
    for _ in range(2):
        o = torch.full((96, 160), complex(np.nan, np.nan), dtype=torch.complex64, device=cuda)
        st = lib.tg_field_direct_noalloc(C.byref(m), C.byref(beams.struct()), C.byref(pm),
                                         torch.view_as_real(o).data_ptr(), N.stream_ptr())
        assert st == 0, st
        outs.append(o)
    torch.cuda.synchronize()
    r = ref.cpu().numpy()
    for o in outs:
        g = o.cpu().numpy()
        assert np.isfinite(g).all()
        assert np.max(np.abs(g - r)) / np.max(np.abs(r)) <= TOL
    assert torch.equal(outs[0], outs[1])
    assert N.error_word() == 0
    # and directly against the float64 oracle on a pixel sample
    import oracle.field as OF
    idx = np.random.default_rng(1).choice(96 * 160, 256, replace=False)
    ref_o = OF.make_gaussian_image(w["rays"], w["model"], pixel_index=idx, chunk=1024)
    g0 = outs[0].cpu().numpy().reshape(-1)[idx]
    assert np.max(np.abs(g0 - ref_o)) / np.max(np.abs(ref_o)) <= 1e-4
    del keep


def test_noalloc_rejects_sizes_beyond_its_limits(cuda):
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300 import gaussian as G
    lib = _lib()
    m = N.TgModel()
    m.n_components = 0
    b = G.TgBeams()
    b.n = 32769  # beyond the 32768-beam maximum
    pm = G.TgPixelMap()
    pm.h, pm.w = 64, 64
    out = torch.empty((64, 64), dtype=torch.complex64, device=cuda)
    assert lib.tg_field_direct_noalloc(C.byref(m), C.byref(b), C.byref(pm),
                                       torch.view_as_real(out).data_ptr(), None) == -5
    b.n = 16
    pm.h, pm.w = 4096, 4096  # one partial image alone exceeds the scratch
    assert lib.tg_field_direct_noalloc(C.byref(m), C.byref(b), C.byref(pm),
                                       torch.view_as_real(out).data_ptr(), None) == -5


def test_noalloc_at_its_size_limit(cuda):
    """The largest image the array holds for 2,000 beams (1800 columns): one
    partial image fills it, so every beam is summed in a single chunk (the
    regular path uses many); one more row is rejected."""
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.gaussian import BeamSet, pixel_map
    from temgymcore_gb300.run import pack_model
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    lib = _lib()
    n, wd = 2000, 1800
    h = _max_rows(n, wd)
    assert _part(n) + 8 * h * wd <= SCRATCH < _part(n) + 8 * (h + 1) * wd
    w = beamlet_field(seed=5, n_beams=n, det_shape=(h, wd), det_px=3e-5, astigmatic=True)
    rays, comps = gaussian_rays(w["rays"]), build_model(w["model"])
    ref = t.FieldPlan(rays, comps, method="direct").evaluate("direct").clone()
    beams = BeamSet(rays, cuda)
    pm = pixel_map(comps[-1])
    m, keep = pack_model(comps)
    o = torch.full((h, wd), complex(np.nan, np.nan), dtype=torch.complex64, device=cuda)
    for _ in range(2):
        st = lib.tg_field_direct_noalloc(C.byref(m), C.byref(beams.struct()), C.byref(pm),
                                         torch.view_as_real(o).data_ptr(), N.stream_ptr())
        assert st == 0, st
        torch.cuda.synchronize()
        g, r = o.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(g).all()
        assert np.max(np.abs(g - r)) / np.max(np.abs(r)) <= TOL
    w2 = beamlet_field(seed=5, n_beams=n, det_shape=(h + 1, wd), det_px=3e-5, astigmatic=True)
    comps2 = build_model(w2["model"])
    pm2 = pixel_map(comps2[-1])
    m2, keep2 = pack_model(comps2)
    big = torch.empty((h + 1, wd), dtype=torch.complex64, device=cuda)
    assert lib.tg_field_direct_noalloc(C.byref(m2), C.byref(beams.struct()), C.byref(pm2),
                                       torch.view_as_real(big).data_ptr(), N.stream_ptr()) == -5
    assert N.error_word() == 0
    del keep, keep2
