"""The batched sweep's host planner (tg_batch_plan, CPU only): the tile table
hands out the longest tiles first, and every model's tiles cover its rays
exactly once with slots 0..n-1 (the per-model partials reduce in slot order,
so the result does not depend on which CTA took which tile)."""
import ctypes as C

import numpy as np

TILE = np.dtype([("model", "<i4"), ("count", "<i4"), ("start", "<i8"), ("slot", "<i4"), ("pad", "<i4")])
HEADER = np.dtype([("n_models", "<i4"), ("n_tiles", "<i4"), ("total_steps", "<i4"), ("tile_rays", "<i4"),
                   ("models_off", "<i8"), ("tiles_off", "<i8"), ("ops_off", "<i8"), ("mom_model_off", "<i8"),
                   ("partial_doubles", "<i8"), ("moment_doubles", "<i8")])


def _plan(specs, counts, tile_rays):
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import TgBatchInfo
    from temgymcore_gb300.run import pack_model
    from temgymcore_gb300.workloads import build_model
    packed = [pack_model(build_model(s)) for s in specs]
    arr = (N.TgModel * len(specs))()
    for i, (m, _) in enumerate(packed):
        arr[i] = m
    cnt = (C.c_int64 * len(specs))(*[int(c) for c in counts])
    info = TgBatchInfo()
    assert N.lib().tg_batch_plan(len(specs), arr, cnt, None, tile_rays, None, 0, C.byref(info)) == 0
    host = np.zeros(info.plan_bytes, dtype=np.uint8)
    assert N.lib().tg_batch_plan(len(specs), arr, cnt, None, tile_rays, host.ctypes.data, host.nbytes,
                                 C.byref(info)) == 0
    hdr = np.frombuffer(host[:HEADER.itemsize].tobytes(), dtype=HEADER)[0]
    off = int(hdr["tiles_off"])
    tiles = np.frombuffer(host[off:off + TILE.itemsize * int(hdr["n_tiles"])].tobytes(), dtype=TILE)
    del packed
    return info, hdr, tiles


def test_tiles_longest_first_and_cover_each_model_once():
    from temgymcore_gb300.workloads import batched_sweep
    w = batched_sweep(seed=3, n_models=48)
    counts = np.asarray(w["counts"], dtype=np.int64).copy()
    counts[5] = 0            # an empty model still gets one (empty) tile
    counts[7] = 4096         # exactly one full tile
    tile_rays = 4096
    info, hdr, tiles = _plan(w["specs"], counts, tile_rays)
    assert int(hdr["n_tiles"]) == info.n_tiles == tiles.size
    assert int(hdr["tile_rays"]) == tile_rays
    ncomp = np.array([len(s) for s in w["specs"]])
    # work = rays x (components + adjoint overhead), non-increasing along the table
    work = tiles["count"].astype(np.int64) * (ncomp[tiles["model"]] + 2)
    assert np.all(np.diff(work) <= 0)
    offsets = np.concatenate([[0], np.cumsum(counts)])
    for m in range(len(w["specs"])):
        t = tiles[tiles["model"] == m]
        n_tiles = max(1, -(-int(counts[m]) // tile_rays))
        assert t.size == n_tiles, m
        assert sorted(t["slot"].tolist()) == list(range(n_tiles)), m
        assert int(t["count"].sum()) == int(counts[m]), m
        assert np.all(t["count"] <= tile_rays)
        np.testing.assert_array_equal(t["start"], offsets[m] + t["slot"].astype(np.int64) * tile_rays)
    assert int(info.total_rays) == int(counts.sum())
