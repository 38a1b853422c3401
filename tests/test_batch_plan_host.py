"""The batched sweep's host planner (tg_batch_plan, CPU only): the tile table
hands out the longest tiles first, and every model's tiles cover its rays
exactly once with slots 0..n-1 (the per-model partials reduce in slot order,
so the result does not depend on which CTA took which tile); each model's
composed output map and its per-step-sum coefficients, contracted with
moments formed on the CPU, reproduce the oracle's outputs and reverse-mode
per-step sums."""
import ctypes as C

import numpy as np

TILE = np.dtype([("model", "<i4"), ("count", "<i4"), ("start", "<i8"), ("slot", "<i4"), ("pad", "<i4")])
HEADER = np.dtype([("n_models", "<i4"), ("n_tiles", "<i4"), ("total_steps", "<i4"), ("tile_rays", "<i4"),
                   ("models_off", "<i8"), ("tiles_off", "<i8"), ("ops_off", "<i8"), ("mom_model_off", "<i8"),
                   ("rec_off", "<i8"), ("coef_off", "<i8"), ("partial_doubles", "<i8"), ("moment_doubles", "<i8")])
MODEL = np.dtype([("op_off", "<i4"), ("n_steps", "<i4"), ("n_tiles", "<i4"), ("n_ev", "<i4"),
                  ("ray_off", "<i8"), ("n_rays", "<i8"), ("pl_const", "<f8"), ("z_out", "<f8"),
                  ("part_off", "<i8"), ("n_bip", "<i4"), ("n_mom", "<i4"), ("mom_off", "<i8"),
                  ("coef_off", "<i8"), ("rec_off", "<i8"), ("rec_floats", "<i4"), ("ev_off", "<i4")])


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
    _plan.host = host
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


def _eval_record(rec, nb, n_ev, ev_off, v):
    """NumPy float64 evaluation of one model's forward record (the kernel's
    closed forms): outputs, the per-ray pathlength part, alive, signs."""
    D = 5 + nb
    D4 = (D + 3) & ~3
    q0 = 4 * D
    l0 = q0 + 16
    k0 = l0 + 8 * nb
    n = v[0].size
    s = np.zeros((nb, n))
    alive = np.ones(n, bool)
    e = ev_off

    def dot(row, nbs):
        acc = row[4] + sum(row[c] * v[c] for c in range(4))
        return acc + sum(row[5 + b] * s[b] for b in range(nbs))
    nbs = 0
    for _ in range(n_ev):
        kind, slot = rec[e:e + 2].view(np.int32)
        r2, cx, cy = rec[e + 2:e + 5].astype(np.float64)
        xr = rec[e + 8:e + 8 + D].astype(np.float64)
        if kind == 0:
            s[slot] = np.sign(dot(xr, nbs))
            nbs += 1
            e += 8 + D4
        else:
            yr = rec[e + 8 + D4:e + 8 + D4 + D].astype(np.float64)
            alive &= dot(xr, nbs) ** 2 + dot(yr, nbs) ** 2 < r2  # the rows hold x - cx, y - cy
            e += 8 + 2 * D4
    cols = rec[:4 * D].astype(np.float64).reshape(D, 4)
    u = np.vstack(list(v) + [np.ones(n)] + list(s))
    out = cols.T @ u
    q = rec[q0:q0 + 16].astype(np.float64)
    p = sum(q[1 + i] * v[i] for i in range(4))
    qi = 5
    for i in range(4):
        for j in range(i, 4):
            p = p + q[qi] * v[i] * v[j]
            qi += 1
    for b in range(nb):
        lb = rec[l0 + 8 * b:l0 + 8 * b + 5].astype(np.float64)
        kb = rec[k0 + b * nb - (b * (b - 1)) // 2:].astype(np.float64)
        lin = lb[4] + sum(lb[c] * v[c] for c in range(4)) + sum(kb[b2 - b] * s[b2] for b2 in range(b, nb))
        p = p + s[b] * lin
    return out, p, alive, s


def test_composed_map_and_step_coefficients_match_the_oracle():
    from oracle.adjoint import forward_tape, value_and_raw
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import batched_sweep
    w = batched_sweep(seed=11, n_models=24, rays=(200, 600))
    # one model with every linear kind, two biprisms and an off-centre aperture
    w["specs"][0] = [{"kind": "scanner", "z": 0.01, "scan_pos_x": 2e-4, "scan_pos_y": -1e-4},
                     {"kind": "lens", "z": 0.05, "focal_length": 0.03},
                     {"kind": "biprism", "z": 0.08, "def_x": 1e-3},
                     {"kind": "rotator", "z": 0.1, "angle": 31.0},
                     {"kind": "deflector", "z": 0.12, "def_x": 3e-4, "def_y": -2e-4},
                     {"kind": "biprism", "z": 0.15, "def_x": -2e-3},
                     {"kind": "aperture", "z": 0.2, "radius": 4e-3, "centre": (5e-4, -2e-4)},
                     {"kind": "lens", "z": 0.25, "focal_length": 0.5}]
    info, hdr, _ = _plan(w["specs"], w["counts"], 4096)
    host = _plan.host
    mods = np.frombuffer(host[int(hdr["models_off"]):int(hdr["models_off"]) + MODEL.itemsize * len(w["specs"])]
                         .tobytes(), dtype=MODEL)
    recs = np.frombuffer(host[int(hdr["rec_off"]):int(hdr["coef_off"])].tobytes(), dtype="<f4")
    coef = np.frombuffer(host[int(hdr["coef_off"]):].tobytes(), dtype="<f8")
    off = np.concatenate([[0], np.cumsum(w["counts"])])
    n_blocked = 0
    for m, spec in enumerate(w["specs"]):
        M = mods[m]
        sl = slice(off[m], off[m + 1])
        v = [w[k][sl].astype(np.float64) for k in ("x", "y", "dx", "dy")]
        t = [w[k][sl].astype(np.float64) for k in ("tx", "ty")]
        tape, ref = forward_tape(ORay(*v, z=np.asarray(0.0), pathlength=np.asarray(0.0)), spec)
        signs = [np.sign(r.x) for step, _, r in tape if step != "free" and step["kind"] == "biprism"]
        nb, nm, ns = int(M["n_bip"]), int(M["n_mom"]), int(M["n_steps"])
        assert nb == len(signs) and nm == 11 + 2 * nb and ns == 2 * len(spec)
        rec = recs[int(M["rec_off"]):int(M["rec_off"]) + int(M["rec_floats"])]
        out, p, alive, s = _eval_record(rec, nb, int(M["n_ev"]), int(M["ev_off"]), v)
        for b in range(nb):
            assert np.array_equal(s[b], signs[b]), (m, b)
        for k, row in zip(("x", "y", "dx", "dy"), out):
            r = getattr(ref, k)
            assert np.max(np.abs(row - r)) <= 2e-7 * np.max(np.abs(r)), (m, k)
        pl = M["pl_const"] + p
        assert np.max(np.abs(pl - ref.pathlength)) <= 5e-9 * np.max(np.abs(ref.pathlength)), m
        ra = np.ones(v[0].size, bool) if ref.alive is None else ref.alive
        assert np.array_equal(alive, ra), m
        n_blocked += int((~ra).sum())
        lx = np.where(ra, 2 * (ref.x - t[0]), 0.0)
        ly = np.where(ra, 2 * (ref.y - t[1]), 0.0)
        vv = np.stack(v + [np.ones_like(v[0])])
        mom = np.zeros(nm)
        for a, la in enumerate((lx, ly)):
            mom[5 * a:5 * a + 5] = vv @ la
            for b, sg in enumerate(signs):
                mom[11 + 2 * b + a] = np.sum(sg * la)
        mom[10] = np.sum((lx * lx + ly * ly) / 4)
        cf = coef[int(M["coef_off"]):int(M["coef_off"]) + ns * 4 * nm].reshape(ns, 4, nm)
        loss, raw, _ = value_and_raw(spec, *v, *t)
        np.testing.assert_allclose(cf @ mom, raw, rtol=0, atol=1e-10 * np.max(np.abs(raw)))
        assert np.isclose(mom[10], loss, rtol=1e-12)
    assert n_blocked > 0
