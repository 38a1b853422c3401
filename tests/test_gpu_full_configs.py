"""Full-size parity through size-independent properties, at the sizes the
benchmarks run: the 4D-STEM scan (64 x 64 probes x 1,024 rays, 256 x 256
images) and the 512-model batched sweep (~23.5 M rays).  The oracle is too
slow for every probe or model, so each test checks invariants on the whole
output and the oracle on a seeded sample."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu


def test_stem_full_scan_properties(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.workloads import stem_4d, stem_model, stem_probe_model
    w = stem_4d(seed=0)
    model = stem_model(w)
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                z=0.0, pathlength=0.0)
    imgs, xy = t.scan_images(ray, model, return_xy=True)
    n_probes, n = xy.shape[0], xy.shape[2]
    assert imgs.shape == (4096, 256, 256) and n == 1024
    # 1. every image holds exactly the in-bounds hits of its probe, binned by
    #    a separate kernel (tg_bin) from the scan's own detector coordinates
    det = model[-1]
    g = det._tg_grid()
    fx = xy[:, 0].contiguous().reshape(-1)
    fy = xy[:, 1].contiguous().reshape(-1)
    py = torch.empty(fx.numel(), dtype=torch.int32, device=cuda)
    px = torch.empty_like(py)
    N.check(N.lib().tg_bin(fx.numel(), N.ptr(fx), N.ptr(fy), None, C.byref(g), N.ptr(py), N.ptr(px),
                           None, 0, N.stream_ptr()), "tg_bin")
    inb = ((py >= 0) & (py < 256) & (px >= 0) & (px < 256)).reshape(n_probes, n)
    assert torch.equal(imgs.sum(dim=(1, 2), dtype=torch.int64), inb.sum(dim=1, dtype=torch.int64))
    assert int(imgs.min()) >= 0
    # 2. a seeded sample of probes: coordinates and images against the oracle
    pos = t.scan_positions(model[1])
    gd = {k: w["detector"][k] for k in ("pixel_size", "shape")}
    for p in np.random.default_rng(1).choice(n_probes, 8, replace=False):
        spx, spy = pos[p]
        ref = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], w["z"], 0.0),
                                stem_probe_model(w, spx, spy))
        gx = xy[p, 0].cpu().numpy().astype(np.float64)
        gy = xy[p, 1].cpu().numpy().astype(np.float64)
        assert normwise_err(gx, ref.x) <= 1e-6 and normwise_err(gy, ref.y) <= 1e-6, p
        opy, opx = oracle.metres_to_pixels(gd, gx, gy)
        assert np.array_equal(imgs[p].cpu().numpy(), oracle.into_image(gd, opy, opx).astype(np.int32)), p
    # 3. the launch is deterministic
    assert torch.equal(t.scan_images(ray, model), imgs)
    assert N.error_word() == 0


def test_batched_full_sweep_properties(cuda):
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import batched_sweep, build_model
    w = batched_sweep(seed=0)
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=16384)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out, raw = bt.alloc_outputs(), bt.alloc_raw()
    bt.run(x, y, dx, dy, out, (tx, ty), raw, 256, 2)
    out2, raw2 = bt.alloc_outputs(), bt.alloc_raw()
    bt.run(x, y, dx, dy, out2, (tx, ty), raw2, 256, 2)
    torch.cuda.synchronize()
    # 1. deterministic across launches (tiles taken by different CTAs)
    assert all(torch.equal(a, b) for a, b in zip(out, out2)) and torch.equal(raw, raw2)
    assert all(bool(torch.isfinite(o).all()) for o in out)
    # 2. a seeded sample of models (up to ~50k rays each) against the oracle
    #    and against the generic per-model adjoint
    rng = np.random.default_rng(2)
    small = [m for m in range(len(models)) if 0 < int(w["counts"][m]) <= 50_000]
    for m in rng.choice(small, 6, replace=False):
        a, b = int(bt.offsets[m]), int(bt.offsets[m + 1])
        ref = oracle.run_to_end(ORay.from_f32(w["x"][a:b], w["y"][a:b], w["dx"][a:b], w["dy"][a:b], 0.0, 0.0),
                                w["specs"][m])
        for k, o in zip(("x", "y", "dx", "dy"), out[:4]):
            assert normwise_err(o[a:b].cpu().numpy(), getattr(ref, k)) <= 5e-6, (m, k)
        mm, keep = pack_model(models[m])
        n = b - a
        gx = (2 * (out[0][a:b] - tx[a:b])).contiguous()
        gy = (2 * (out[1][a:b] - ty[a:b])).contiguous()
        z = torch.zeros(n, device=cuda)
        r2 = torch.zeros((2 * len(models[m]), 4), dtype=torch.float64, device=cuda)
        ws = torch.empty(max(8, N.lib().tg_trace_vjp_workspace(n, C.byref(mm))), dtype=torch.uint8,
                         device=cuda)
        xs = [v[a:b].contiguous() for v in (x, y, dx, dy)]
        rin = _rays_struct(n, *xs, None, 0.0, None, 0.0)
        gout = _rays_struct(n, gx, gy, z, z, None, 0.0, None, 0.0)
        N.check(N.lib().tg_trace_vjp(C.byref(mm), C.byref(rin), C.byref(gout), None, r2.data_ptr(),
                                     ws.data_ptr(), ws.numel(), N.stream_ptr()))
        assert normwise_err(bt.model_raw(raw, m).cpu().numpy(), r2.cpu().numpy()) <= 1e-4, m
        del keep
    assert N.error_word() == 0
