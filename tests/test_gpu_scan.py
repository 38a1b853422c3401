"""GPU parity of the 4D-STEM scan batch (per-probe dense histograms)."""
import numpy as np
import pytest
import torch

import oracle
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu


def np_(t):
    return t.detach().cpu().numpy()


def _check(w, imgs, xy, positions):
    from temgymcore_gb300.workloads import stem_probe_model
    g = {k: w["detector"][k] for k in ("pixel_size", "shape")}
    n = w["x"].size
    for p in range(imgs.shape[0]):
        spx, spy = positions[p]
        spec = stem_probe_model(w, spx, spy)
        ref = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], w["z"], 0.0), spec)
        gx, gy = np_(xy[p, 0]), np_(xy[p, 1])
        assert normwise_err(gx, ref.x) <= 1e-6 and normwise_err(gy, ref.y) <= 1e-6, p
        py, px = oracle.metres_to_pixels(g, gx.astype(np.float64), gy.astype(np.float64))
        acc = oracle.into_image(g, py, px).astype(np.int32)
        assert np.array_equal(np_(imgs[p]), acc), p
        assert int(acc.sum()) <= n


def test_stem_small_scan_matches_oracle(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_4d, stem_model
    w = stem_4d(seed=0, scan=(6, 5), rays_per_probe=1024)
    model = stem_model(w)
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                z=0.0, pathlength=0.0)
    imgs, xy = t.scan_images(ray, model, return_xy=True)
    assert imgs.shape == (30, 256, 256)
    pos = t.scan_positions(model[1])
    # scan positions follow the ScanGrid map (oracle restatement)
    sg = {k: w["scangrid"][k] for k in ("pixel_size", "shape", "rotation")}
    yy, xx = np.meshgrid(np.arange(6), np.arange(5), indexing="ij")
    ox, oy = oracle.pixels_to_metres(sg, yy.ravel(), xx.ravel())
    np.testing.assert_array_equal(pos[:, 0], ox)
    np.testing.assert_array_equal(pos[:, 1], oy)
    _check(w, imgs, xy, pos)
    # images without the coordinate side output are identical
    assert torch.equal(t.scan_images(ray, model), imgs)
    assert t._native.error_word() == 0


def test_stem_explicit_positions_wide_spread_and_big_bundle(cuda):
    """Slow paths: a spread too wide for the shared window, and a bundle too
    large for the shared pixel buffer; plus explicit positions."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_4d, stem_model
    for rays, semi in ((1024, 4e-1), (5000, 5e-3)):
        w = stem_4d(seed=3, scan=(2, 3), rays_per_probe=rays, semi_conv=semi)
        model = stem_model(w)
        rng = np.random.default_rng(4)
        pos = rng.normal(0, 2e-4, (7, 2))
        ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                    dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                    z=0.0, pathlength=0.0)
        imgs, xy = t.scan_images(ray, model, positions=pos, return_xy=True)
        _check(w, imgs, xy, pos)


def test_stem_empty_cases(cuda):
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_4d, stem_model
    w = stem_4d(seed=1, scan=(2, 2), rays_per_probe=8)
    model = stem_model(w)
    e = torch.empty(0, device=cuda)
    imgs = t.scan_images(t.Ray(x=e, y=e, dx=e, dy=e, z=0.0, pathlength=0.0), model)
    assert imgs.shape == (4, 256, 256) and int(imgs.abs().sum()) == 0
    imgs = t.scan_images(t.Ray(x=e, y=e, dx=e, dy=e, z=0.0, pathlength=0.0), model,
                         positions=np.zeros((0, 2)))
    assert imgs.shape == (0, 256, 256)


def test_stem_probes_that_miss_and_garbage_output(cuda):
    """Probes whose whole bundle misses the detector (images written only by
    the zero-row copies), probes near the edge (window rows at the image
    border), over an output buffer pre-filled with garbage."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_4d, stem_model
    w = stem_4d(seed=5, scan=(2, 2), rays_per_probe=1024)
    model = stem_model(w)
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                z=0.0, pathlength=0.0)
    half = 0.5 * 256 * w["detector"]["pixel_size"][0]
    pos = np.array([[0.0, 0.0], [1.0, 1.0], [half * 0.98, 0.0], [0.0, -half * 0.98], [-half * 0.97, half * 0.97]])
    out = torch.full((len(pos), 256, 256), 12345, dtype=torch.int32, device=cuda)
    imgs, xy = t.scan_images(ray, model, positions=pos, out=out, return_xy=True)
    _check(w, imgs, xy, pos)
    assert int(imgs[1].abs().sum()) == 0
    assert t._native.error_word() == 0


def test_stem_images_into_pinned_host_memory(cuda):
    """scan_images with a pinned host output (the kernel writes across the
    host link, plain stores instead of the bulk zero rows) equals the device
    result."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_4d, stem_model
    w = stem_4d(seed=6, scan=(3, 4), rays_per_probe=1024)
    model = stem_model(w)
    ray = t.Ray(x=torch.tensor(w["x"], device=cuda), y=torch.tensor(w["y"], device=cuda),
                dx=torch.tensor(w["dx"], device=cuda), dy=torch.tensor(w["dy"], device=cuda),
                z=0.0, pathlength=0.0)
    dev_imgs = t.scan_images(ray, model)
    host = torch.full((12, 256, 256), -7, dtype=torch.int32).pin_memory()
    t.scan_images(ray, model, out=host)
    torch.cuda.synchronize()
    assert torch.equal(host, dev_imgs.cpu())
    with pytest.raises(ValueError):
        t.scan_images(ray, model, out=torch.zeros((12, 256, 256), dtype=torch.int32))
    assert t._native.error_word() == 0
