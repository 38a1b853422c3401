"""Full-size parity at the sizes the benchmarks run: the 4D-STEM scan
(64 x 64 probes x 1,024 rays, 256 x 256 images: invariants on the whole
output and the oracle on a seeded sample of probes) and the 512-model
batched sweep (~23.5 M rays: every model against the oracle)."""
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


def test_batched_full_sweep_every_model(cuda):
    """The 512-model sweep (~23.5 M rays, apertures active): every model's
    coordinates, pathlength and alive mask against the float64 oracle; the
    loss and per-step sums against the oracle's reverse mode for the largest
    models, the deepest models and a seeded sample; repeat launches equal.
    The largest errors are printed (pytest -s)."""
    from test_gpu_batch import check_model

    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.workloads import batched_sweep, build_model
    w = batched_sweep(seed=0)
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=16384)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out, raw, alive, loss = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    bt.run(x, y, dx, dy, out, (tx, ty), raw, 256, 2, alive=alive, loss=loss)
    out2, raw2, alive2, loss2 = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    bt.run(x, y, dx, dy, out2, (tx, ty), raw2, 256, 2, alive=alive2, loss=loss2)
    torch.cuda.synchronize()
    # 1. deterministic across launches (tiles taken by different CTAs)
    assert all(torch.equal(a, b) for a, b in zip(out, out2)) and torch.equal(raw, raw2)
    assert torch.equal(alive, alive2) and torch.equal(loss, loss2)
    assert all(bool(torch.isfinite(o).all()) for o in out)
    n_alive = int(alive.sum())
    assert 0 < n_alive < bt.total  # the apertures block some rays and pass others
    counts = w["counts"]
    depth = np.array([len(s) for s in w["specs"]])
    rng = np.random.default_rng(2)
    adj = set(np.argsort(counts)[-4:]) | set(np.argsort(-depth, kind="stable")[:4])
    adj |= set(rng.choice(len(models), 8, replace=False))
    raw_h, loss_h = raw.cpu().numpy(), loss.cpu().numpy()
    out_h, alive_h = [o.cpu() for o in out], alive.cpu()
    worst = {}
    set_aside = 0
    for m in range(len(models)):
        a, b = int(bt.offsets[m]), int(bt.offsets[m + 1])
        if b == a:
            continue
        if m in adj:
            errs, n_tie = check_model(w, m, a, b, out_h, alive_h, bt.model_raw(raw_h, m), float(loss_h[m]))
        else:  # coordinates only (the adjoint check is the costly part)
            errs, n_tie = _forward_only(w, m, a, b, out_h, alive_h)
        set_aside += n_tie
        for k, v in errs.items():
            worst[k] = max(worst.get(k, 0.0), v)
    print(f"batched sweep: {bt.total} rays ({n_alive} alive), worst normwise errors {worst}, "
          f"{set_aside} rays within 1e-5 of a sign/aperture threshold set aside")
    assert set_aside <= 1e-4 * bt.total
    assert N.error_word() == 0


def _forward_only(w, m, a, b, out, alive):
    from test_gpu_batch import TIE

    from oracle.adjoint import margins
    spec = w["specs"][m]
    sl = slice(a, b)
    f64 = lambda k: w[k][sl].astype(np.float64)  # noqa: E731
    ref = oracle.run_to_end(ORay(f64("x"), f64("y"), f64("dx"), f64("dy"), 0.0, 0.0), spec)
    keep = margins(spec, f64("x"), f64("y"), f64("dx"), f64("dy")) > TIE
    errs = {}
    for k, o in zip(("x", "y", "dx", "dy"), out[:4]):
        errs[k] = normwise_err(o[sl].cpu().numpy()[keep], getattr(ref, k)[keep])
        assert errs[k] <= 1e-6, (m, k, errs[k])
    errs["pathlength"] = normwise_err(out[4][sl].cpu().numpy()[keep], np.broadcast_to(ref.pathlength, keep.shape)[keep])
    assert errs["pathlength"] <= 5e-7, m
    ra = np.ones(b - a, bool) if ref.alive is None else ref.alive
    assert np.array_equal(alive[sl].cpu().numpy()[keep].astype(bool), ra[keep]), m
    return errs, int((~keep).sum())
