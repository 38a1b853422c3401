"""Batched persistent launch (forward + adjoint of the squared-residual loss)
against the float64 oracle per model.

Bounds: coordinates <= 1e-6 normwise per model and field; pathlength <= 5e-7
normwise (the per-ray part is evaluated in float32, and behind two 1 cm
lenses it reaches the order of the whole pathlength); the alive mask equal; per-step sums and loss <= 1e-5 normwise
against the oracle's reverse-mode value-and-gradient (oracle/adjoint.py),
which is itself pinned to complex-step derivatives on the CPU.  Rays whose
biprism sign or aperture test lies within 1e-5 (relative) of its threshold
in the float64 chain are set aside from the per-ray comparisons: there the
float32 decision may round the other way."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from oracle.adjoint import complex_step_grads, margins, param_grads, value_and_raw
from oracle.rays import ORay
from conftest import normwise_err

pytestmark = pytest.mark.gpu

TIE = 1e-5


def _small(seed=1):
    from temgymcore_gb300.workloads import batched_sweep
    w = batched_sweep(seed=seed, n_models=24, rays=(1, 3000))
    off = np.concatenate([[0], np.cumsum(w["counts"])])
    cut = np.arange(off[3], off[4])
    w["counts"] = w["counts"].copy()
    w["counts"][3] = 0  # an empty model
    for k in ("x", "y", "dx", "dy", "tx", "ty"):
        w[k] = np.delete(w[k], cut)
    return w


def check_model(w, m, a, b, out, alive, raw_m, loss_m, tol_xy=1e-6, tol_adj=1e-5):
    """Compare one model's batched results with the oracle; returns the
    errors and the number of rays set aside."""
    spec = w["specs"][m]
    sl = slice(a, b)
    f64 = lambda k: w[k][sl].astype(np.float64)  # noqa: E731
    ref = oracle.run_to_end(ORay(f64("x"), f64("y"), f64("dx"), f64("dy"), 0.0, 0.0), spec)
    keep = margins(spec, f64("x"), f64("y"), f64("dx"), f64("dy")) > TIE
    errs = {}
    for k, o in zip(("x", "y", "dx", "dy"), out[:4]):
        g = o[sl].cpu().numpy()
        errs[k] = normwise_err(g[keep], getattr(ref, k)[keep])
        assert errs[k] <= tol_xy, (m, k, errs[k])
    errs["pathlength"] = normwise_err(out[4][sl].cpu().numpy()[keep], np.broadcast_to(ref.pathlength, keep.shape)[keep])
    assert errs["pathlength"] <= 5e-7, (m, errs["pathlength"])
    ra = np.ones(b - a, bool) if ref.alive is None else ref.alive
    assert np.array_equal(alive[sl].cpu().numpy()[keep].astype(bool), ra[keep]), m
    loss, raw, _ = value_and_raw(spec, f64("x"), f64("y"), f64("dx"), f64("dy"), f64("tx"), f64("ty"))
    errs["raw"] = normwise_err(raw_m, raw)
    errs["loss"] = abs(loss_m - loss) / max(abs(loss), 1e-300)
    if keep.all():
        assert errs["raw"] <= tol_adj, (m, errs["raw"])
        assert errs["loss"] <= tol_adj, (m, errs["loss"])
    return errs, int((~keep).sum())


def test_batched_forward_and_adjoint(cuda):
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.workloads import build_model
    from temgymcore_gb300 import _native as N
    w = _small()
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=512)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out, raw, alive, loss = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    for block, rpt in ((256, 1), (128, 4), (512, 2)):
        raw.zero_()
        bt.run(x, y, dx, dy, out, (tx, ty), raw, block, rpt, alive=alive, loss=loss)
        torch.cuda.synchronize()
        for m in range(len(models)):
            a, b = int(bt.offsets[m]), int(bt.offsets[m + 1])
            if b == a:
                assert np.all(bt.model_raw(raw, m).cpu().numpy() == 0) and float(loss[m]) == 0.0
                continue
            check_model(w, m, a, b, out, alive, bt.model_raw(raw, m).cpu().numpy(), float(loss[m]))
    assert N.error_word() == 0


def test_batched_adjoint_against_complex_step(cuda):
    """Named parameter gradients (z, focal length, deflections) of a few
    models against complex-step derivatives of the oracle's loss."""
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.workloads import build_model
    w = _small(seed=4)
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=1024)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    h_loss, h_raw = bt.value_and_grad(*(torch.from_numpy(w[k]) for k in ("x", "y", "dx", "dy", "tx", "ty")))
    d_loss, d_raw = bt.value_and_grad(x, y, dx, dy, tx, ty)
    torch.cuda.synchronize()
    assert torch.equal(h_raw, d_raw.cpu()) and torch.equal(h_loss, d_loss.cpu())
    checked = 0
    for m in range(len(models)):
        a, b = int(bt.offsets[m]), int(bt.offsets[m + 1])
        spec = w["specs"][m]
        f64 = [w[k][a:b].astype(np.float64) for k in ("x", "y", "dx", "dy", "tx", "ty")]
        if b - a < 50 or not (margins(spec, *f64[:4]) > TIE).all():
            continue
        cs = complex_step_grads(spec, *f64)
        got = bt.grads(h_raw, m)
        scale = max(abs(v) for g in cs for v in g.values())
        for gi, ci in zip(got, cs):
            for k, v in ci.items():
                assert abs(gi[k] - v) <= 1e-5 * scale, (m, k, gi[k], v)
        # the oracle's reverse mode gives the same named gradients
        _, raw_o, _ = value_and_raw(spec, *f64)
        for go, ci in zip(param_grads(spec, raw_o), cs):
            for k, v in ci.items():
                assert abs(go[k] - v) <= 1e-9 * scale
        checked += 1
    assert checked >= 5


def test_batched_matches_generic_adjoint(cuda):
    """Per-step sums equal the per-model generic adjoint (tg_trace_vjp) given
    the upstream gradient 2 (r - target) on alive rays."""
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import build_model
    w = _small(seed=6)
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=512)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out, raw, alive = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive()
    bt.run(x, y, dx, dy, out, (tx, ty), raw, alive=alive)
    torch.cuda.synchronize()
    for m in range(len(models)):
        a, b = int(bt.offsets[m]), int(bt.offsets[m + 1])
        if b == a:
            continue
        mm, keep = pack_model(models[m])
        n = b - a
        al = alive[a:b].to(torch.float32)
        gx = (2 * (out[0][a:b] - tx[a:b]) * al).contiguous()
        gy = (2 * (out[1][a:b] - ty[a:b]) * al).contiguous()
        z = torch.zeros(n, device=cuda)
        r2 = torch.zeros((2 * len(models[m]), 4), dtype=torch.float64, device=cuda)
        ws = torch.empty(max(8, N.lib().tg_trace_vjp_workspace(n, C.byref(mm))), dtype=torch.uint8,
                         device=cuda)
        rin = _rays_struct(n, x[a:b], y[a:b], dx[a:b], dy[a:b], None, 0.0, None, 0.0)
        gout = _rays_struct(n, gx, gy, z, z, None, 0.0, None, 0.0)
        N.check(N.lib().tg_trace_vjp(C.byref(mm), C.byref(rin), C.byref(gout), None, r2.data_ptr(),
                                     ws.data_ptr(), ws.numel(), N.stream_ptr()))
        assert normwise_err(bt.model_raw(raw, m).cpu().numpy(), r2.cpu().numpy()) <= 1e-4, m
        del keep


def test_batched_graph_and_autotune(cuda):
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.workloads import build_model
    w = _small(seed=2)
    bt = BatchedTrace([build_model(s) for s in w["specs"]], w["counts"])
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out = bt.alloc_outputs()
    raw, alive, loss = bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    best, res = bt.autotune(x, y, dx, dy, out, (tx, ty), raw)
    assert best[1] in (128, 256, 512)
    bt.run(x, y, dx, dy, out, (tx, ty), raw, alive=alive, loss=loss)
    ref_raw, ref_x, ref_alive, ref_loss = raw.clone(), out[0].clone(), alive.clone(), loss.clone()
    g = bt.capture(x, y, dx, dy, out, (tx, ty), raw, alive=alive, loss=loss)
    raw.zero_()
    out[0].zero_()
    alive.zero_()
    loss.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out[0], ref_x) and torch.equal(alive, ref_alive)
    assert torch.equal(raw, ref_raw) and torch.equal(loss, ref_loss)  # fixed-order reductions


def test_one_call_batched_trace(cuda):
    """tg_batched_trace (plan + run in one call) equals BatchedTrace.run."""
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace, TgBatchIO
    from temgymcore_gb300.workloads import build_model
    N.register("tg_batched_trace_workspace", C.c_size_t, [C.c_int32, C.POINTER(N.TgModel), C.POINTER(C.c_int64),
                                                          C.POINTER(C.c_double)])
    N.register("tg_batched_trace", C.c_int, [C.c_int32, C.POINTER(N.TgModel), C.POINTER(C.c_int64),
                                             C.POINTER(C.c_double), C.POINTER(TgBatchIO), C.c_void_p, C.c_size_t,
                                             C.c_void_p])
    w = _small(seed=3)
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=4096)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=cuda) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out, raw, alive, loss = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    bt.run(x, y, dx, dy, out, (tx, ty), raw, 256, 2, alive=alive, loss=loss)
    out2, raw2, alive2, loss2 = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    io = bt.io(x, y, dx, dy, out2, (tx, ty), raw2, alive2, loss2)
    cnt = (C.c_int64 * len(models))(*[int(v) for v in w["counts"]])
    nb = N.lib().tg_batched_trace_workspace(len(models), bt._arr, cnt, None)
    assert nb > 0
    ws = torch.empty(nb + 256, dtype=torch.uint8, device=cuda)
    wp = ws.data_ptr() + (-ws.data_ptr()) % 256
    N.check(N.lib().tg_batched_trace(len(models), bt._arr, cnt, None, C.byref(io), wp, nb, N.stream_ptr()))
    torch.cuda.synchronize()
    for a, b in zip(out, out2):
        assert torch.equal(a, b)
    assert torch.equal(raw, raw2) and torch.equal(alive, alive2) and torch.equal(loss, loss2)


def test_loss_without_targets_is_rejected(cuda):
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.workloads import build_model
    w = _small(seed=7)
    bt = BatchedTrace([build_model(s) for s in w["specs"]], w["counts"])
    x = torch.tensor(w["x"], device=cuda)
    with pytest.raises(ValueError):
        bt.run(x, x, x, x, bt.alloc_outputs(), loss=bt.alloc_loss())
