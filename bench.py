"""Benchmark of the GB300 TemGymCore hot path.

Headline workload (one step): the 4D-STEM shadow-image batch - a 64 x 64 scan
(step 1e-9 m, random rotation), one 1,024-ray point-source bundle per probe
(4,194,304 ray traces), descan matrix I + N(0, 1e-3), camera length 0.1 m,
per-probe dense 256 x 256 int32 detector images (1.07 GB written per step).
Metric: ray-component steps per second (rays x components, forward trace +
binning), whole job.  The working set (1.07 GB of images) exceeds the 129 MB
L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs its own scan (weak scaling: probes
are independent, there is no data-path collective); rank 0 prints the line.
``--impl reference`` times the CPU restatement of the reference's per-probe
loop (run_to_end + into_image) on all host cores, same metric and config.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+grad ray·component steps/s; field beam·px/s at stated err vs the float64 kernel"
UNIT = "ray·component steps/s"
SCAN = (64, 64)
RAYS = 1024
N_COMPONENTS = 5  # PointSource, ScanGrid, Scanner, Descanner, Detector
FALLBACK_HBM_GBS = 6800.0


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), float(p.get("bf16_tflops", 1900.0)), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, 1900.0, "fallback"


def _traffic(name):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh).get(name)
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        time.sleep(0.15)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            time.sleep(0.1)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) >= 7:
                try:
                    rows.append((float(f[0]), float(f[1]), f[2:]))
                except ValueError:
                    pass
        if not rows:
            return None
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for _, _, fl in rows:
            for nm, v in zip(names[1:], fl[1:]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


# ------------------------------------------------------------------ helpers

def _setup_dist(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if args.impl == "gb300":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif args.impl == "gb300":
        torch.cuda.set_device(0)
    return world, rank, local


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(v, world):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _workload():
    from temgymcore_gb300.workloads import stem_4d
    return stem_4d(seed=0, scan=SCAN, rays_per_probe=RAYS)


# ------------------------------------------------------------ CPU baseline

def _cpu_probe_chunk(args):
    """Reference loop restated (oracle): run_to_end + metres_to_pixels +
    into_image per probe.  Returns elapsed seconds for ``probes``."""
    sys.path.insert(0, ROOT)
    import oracle
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import stem_4d, stem_probe_model
    probes, = args
    w = stem_4d(seed=0, scan=SCAN, rays_per_probe=RAYS)
    g = {k: w["detector"][k] for k in ("pixel_size", "shape")}
    sg = {k: w["scangrid"][k] for k in ("pixel_size", "shape", "rotation")}
    t0 = time.perf_counter()
    for p in probes:
        r, c = divmod(int(p), SCAN[1])
        spx, spy = oracle.pixels_to_metres(sg, r, c)
        spec = stem_probe_model(w, float(spx), float(spy))
        out = oracle.run_to_end(ORay(w["x"].astype(np.float64), w["y"].astype(np.float64),
                                     w["dx"].astype(np.float64), w["dy"].astype(np.float64),
                                     0.0, 0.0), spec)
        py, px = oracle.metres_to_pixels(g, out.x, out.y)
        oracle.into_image(g, py, px)
    return time.perf_counter() - t0


def cpu_baseline(sample_probes=SCAN[0] * SCAN[1]):
    """Single-core oracle timing on a bounded sample (rank 0, N=1 only)."""
    el = _cpu_probe_chunk((list(range(sample_probes)),))
    v = sample_probes * RAYS * N_COMPONENTS / el
    return {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{sample_probes} of {SCAN[0] * SCAN[1]} probes x {RAYS} rays, NumPy float64 "
                      "restatement of run_to_end + metres_to_pixels + into_image per probe, 1 thread"}


def headline_config(world: int) -> dict:
    """The headline workload (both arms print this config)."""
    return {"workload": "4D-STEM shadow images: 64x64 scan (step 1e-9 m, rotation "
                        "U(0,2pi)), 1024-ray point-source bundle per probe, descan I+N(0,1e-3), "
                        "camera length 0.1 m, 256x256 int32 images at 5.5e-5 m",
            "rays_per_step": SCAN[0] * SCAN[1] * RAYS, "components": N_COMPONENTS,
            "l2": "no flush: 1.07 GB of images written per step > 129 MB L2",
            "parallelism": f"dp{world} (independent scans per rank)"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    # size each step so the whole --steps/--warmup run stays near a minute
    t_probe = _cpu_probe_chunk((list(range(8)),)) / 8
    per_worker = int(min(SCAN[0] * SCAN[1] // cores, max(1, 60.0 / (args.steps + args.warmup)
                                                          / max(t_probe, 1e-6))))
    per_step = per_worker * cores  # a bounded sample of the 4096-probe scan
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        def step():
            chunks = [(list(range(i * per_worker, (i + 1) * per_worker)),) for i in range(cores)]
            t0 = time.perf_counter()
            pool.map(_cpu_probe_chunk, chunks)
            return time.perf_counter() - t0
        for _ in range(args.warmup):
            step()
        times = [step() for _ in range(args.steps)]
    t = sum(times)
    v = args.steps * per_step * RAYS * N_COMPONENTS / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded), no dataset",
            "config": headline_config(1),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per_step} of 4096 probes per step, {cores} spawn workers"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU arm

def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def secondary_plain(torch, dev):
    """Plain paraxial trace, 65,536 rays: fused trace + pixels + histogram,
    through the public call, through a compiled TracePlan, and replayed as a
    CUDA graph."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, plain_trace
    w = plain_trace(seed=0, n=65536)
    model = build_model(w["model"])
    xs = [torch.tensor(w[k], device=dev) for k in ("x", "y", "dx", "dy")]
    ray = t.Ray(x=xs[0], y=xs[1], dx=xs[2], dy=xs[3], z=0.0, pathlength=0.0)
    acc = torch.zeros((256, 256), dtype=torch.int64, device=dev)
    ms_api = _time(torch, lambda: t.trace_to_image(ray, model, acc=acc), 200)
    plan = t.TracePlan(model, *xs, detector=model[-1], pixels=True)
    ms_plan = _time(torch, plan.run, 200)
    g = plan.capture()
    ms_graph = _time(torch, g.replay, 500)
    n = 65536
    return {"workload": "plain trace 65,536 rays, Lens+Detector 256x256, fused trace+pixels+hist",
            "ms_api_call": ms_api, "ms_trace_plan": ms_plan, "ms_graph_replay": ms_graph,
            "rays_per_s_graph": n / (ms_graph * 1e-3),
            "ray_component_steps_per_s_graph": 2 * n / (ms_graph * 1e-3),
            "achieved_gbs_graph": n * 48 / (ms_graph * 1e-3) / 1e9,
            "note": "3.1 MB per step: launch-latency bound; the API call adds host-side packing"}


def _time(torch, fn, reps):
    a, b = _events(torch)
    fn()
    torch.cuda.synchronize()
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def _field_errors(plan, ref, methods, into):
    """Normwise field error and the phase error at bright pixels (> 25% of the
    peak) of each method against a reference image."""
    scale = np.max(np.abs(ref))
    bright = np.abs(ref) > 0.25 * scale
    for name in methods:
        g = plan.evaluate(name).cpu().numpy().astype(np.complex128)
        ph = float(np.max(np.abs(np.angle(g[bright] * np.conj(ref[bright]))))) if bright.any() else None
        into[name].update({"field_rel_err_vs_fp64_kernel": float(np.max(np.abs(g - ref)) / scale),
                           "phase_err_rad_bright": ph})


def secondary_input_field(torch, dev, bf16):
    """Input-plane beamlet field (evaluate_gaussian_input_image): 16,384
    overlapping beams on 512 x 512 pixels; separable split-BF16 GEMM and the
    fast direct kernel (astigmatic beams), errors against the float64 kernel."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import build_model, gaussian_rays, input_field
    w = input_field(seed=0)
    grid = build_model([w["grid"]])[0]
    pairs = 16384 * 512 * 512
    plan = t.FieldPlan(gaussian_rays(w["rays"]), None, grid=grid)
    res = {"workload": f"16,384 beams on a golden-angle spiral (waist {w['waist']:.3g} m, lambda 500 nm, "
                       "slopes N(0,1e-4)), their own plane sampled on 512x512 pixels of 1e-5 m",
           "separable": plan.separable}
    ms_sep = _time(torch, lambda: plan.evaluate("separable"), 20)
    ms_dir = _time(torch, lambda: plan.evaluate("direct"), 3)
    gemm_flops = 12 * 2 * 512 * 512 * 16416
    res["separable_gemm"] = {"ms": ms_sep, "beam_px_per_s": pairs / (ms_sep * 1e-3),
                             "frac_of_bf16_peak": gemm_flops / (ms_sep * 1e-3) / 1e12 / bf16}
    res["direct_fast"] = {"ms": ms_dir, "beam_px_per_s": pairs / (ms_dir * 1e-3)}
    ref = plan.evaluate("fp64").clone().cpu().numpy().astype(np.complex128)
    _field_errors(plan, ref, ("separable", "direct"),
                  {"separable": res["separable_gemm"], "direct": res["direct_fast"]})
    wa = input_field(seed=0, astigmatic=True)
    pa = t.FieldPlan(gaussian_rays(wa["rays"]), None, grid=grid)
    ms_a = _time(torch, lambda: pa.evaluate("direct"), 3)
    res["astigmatic_direct"] = {"ms": ms_a, "beam_px_per_s": pairs / (ms_a * 1e-3), "separable": pa.separable}
    return res


def secondary_field(torch, dev, hbm, bf16):
    """Gaussian-beamlet field, 16,384 beams on 512 x 512 pixels: separable
    split-BF16 tensor-core GEMM, fast direct kernel (astigmatic beams) and the
    all-float64 direct kernel; errors of the fast paths against the float64
    kernel's image (exact k*pl reduction)."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
    res = {"workload": "16,384 beamlets (aperture decomposition, waist 1e-9 m, lambda 1.97e-12 m, "
                       "pl 1 m + N(0,1e-6)), Lens f=0.5 m, 512x512 detector at 1e-5 m"}
    pairs = 16384 * 512 * 512
    w = beamlet_field(seed=0)
    plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
    res["separable"] = plan.separable
    ms_prep = _time(torch, lambda: t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]),
                                               method="separable"), 3)
    ms_sep = _time(torch, lambda: plan.evaluate("separable"), 20)
    ms_dir = _time(torch, lambda: plan.evaluate("direct"), 3)
    ms_f64 = _time(torch, lambda: plan.evaluate("fp64"), 1)
    gemm_flops = 12 * 2 * 512 * 512 * 16416
    res["separable_gemm"] = {"ms": ms_sep, "beam_px_per_s": pairs / (ms_sep * 1e-3),
                             "bf16_issued_tflops": gemm_flops / (ms_sep * 1e-3) / 1e12,
                             "useful_complex_tflops": 8 * pairs / (ms_sep * 1e-3) / 1e12,
                             "frac_of_bf16_peak": gemm_flops / (ms_sep * 1e-3) / 1e12 / bf16,
                             "note": "includes operand generation and split-K reduction"}
    res["direct_fast"] = {"ms": ms_dir, "beam_px_per_s": pairs / (ms_dir * 1e-3)}
    res["direct_fp64"] = {"ms": ms_f64, "beam_px_per_s": pairs / (ms_f64 * 1e-3)}
    res["speedup_separable_vs_fp64"] = ms_f64 / ms_sep
    res["prep_plan_ms"] = ms_prep
    # errors against the all-float64 kernel's image (that kernel is held to
    # 5e-7 of the float64 oracle by the tests; the bench itself runs no oracle)
    ref = plan.evaluate("fp64").clone().cpu().numpy().astype(np.complex128)
    _field_errors(plan, ref, ("separable", "direct"),
                  {"separable": res["separable_gemm"], "direct": res["direct_fast"]})
    # astigmatic case (direct kernel only)
    wa = beamlet_field(seed=0, astigmatic=True)
    pa = t.FieldPlan(gaussian_rays(wa["rays"]), build_model(wa["model"]))
    ms_a = _time(torch, lambda: pa.evaluate("direct"), 3)
    res["astigmatic_direct"] = {"ms": ms_a, "beam_px_per_s": pairs / (ms_a * 1e-3), "separable": pa.separable}
    return res


def secondary_fit(torch, dev):
    """Adjoint fit: 32x32 scan x 1,024 rays, 21 parameters; fused loss +
    gradient + Adam replayed as a CUDA graph, 200 steps; versus the plain
    per-model path (one generic forward + adjoint launch pair per probe)."""
    import ctypes as C

    import temgymcore_gb300 as t
    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.fit import StemFit
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import stem_fit
    w = stem_fit(seed=0)
    ray = t.Ray(x=w["x"], y=w["y"], dx=w["dx"], dy=w["dy"], z=0.0, pathlength=0.0)
    fit = StemFit(ray, w["rows"], w["cols"], w["gap"], w["theta0"])
    fit.set_targets(w["theta_true"])
    sc = np.abs(w["theta0"])
    sc[sc < 1e-2] = 1e-3
    fit.scale.copy_(torch.as_tensor(sc))
    n_probes, n = fit.n_probes, fit.n
    ms_lg = _time(torch, fit.loss_grad, 50)
    fit.capture(1e-3)
    a, b = _events(torch)
    l0 = float(fit.loss_grad()[0])
    torch.cuda.synchronize()
    a.record()
    for _ in range(200):
        fit.graph.replay()
    b.record()
    torch.cuda.synchronize()
    ms_step = a.elapsed_time(b) / 200
    l1 = float(fit.loss_grad()[0])
    th = fit.theta.cpu().numpy()
    rel = np.abs(th[:3] - w["theta_true"][:3]) / np.abs(w["theta_true"][:3])
    # plain per-model path on a sample of probes: tg_trace_fwd + residual + tg_trace_vjp
    sample = 64
    sp = t.scan_positions(fit.model_at(w["theta0"])[1])
    models = [pack_model(fit.model_at(w["theta0"], *sp[p])) for p in range(sample)]
    xs = [as_t.contiguous() for as_t in (fit.x, fit.y, fit.dx, fit.dy)]
    outs = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(4)]
    opl = torch.empty(n, dtype=torch.float64, device=dev)
    g = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(4)]
    ws = torch.empty(1 << 20, dtype=torch.uint8, device=dev)
    raw = torch.zeros((12, 4), dtype=torch.float64, device=dev)
    rin = _rays_struct(n, *xs, None, 0.0, None, 0.0)
    rout = _rays_struct(n, *outs, None, 0.0, opl, 0.0)
    gout = _rays_struct(n, *g, None, 0.0, None, 0.0)
    lib = N.lib()

    def plain():
        for p in range(sample):
            m, _ = models[p]
            lib.tg_trace_fwd(C.byref(m), C.byref(rin), C.byref(rout), None, None, None, None, None, 0,
                             N.stream_ptr())
            torch.sub(outs[0], fit.tx[p], out=g[0]).mul_(2.0)
            torch.sub(outs[1], fit.ty[p], out=g[1]).mul_(2.0)
            g[2].zero_()
            g[3].zero_()
            lib.tg_trace_vjp(C.byref(m), C.byref(rin), C.byref(gout), None, raw.data_ptr(), ws.data_ptr(),
                             ws.numel(), N.stream_ptr())
    ms_plain = _time(torch, plain, 3) * n_probes / sample
    return {"workload": "adjoint fit: 32x32 scan x 1,024 rays (1,048,576 rays), 21 parameters, "
                        "loss = sum of squared detector residuals",
            "loss_grad_ms": ms_lg, "adam_step_graph_ms": ms_step,
            "grad_evals_per_s": 1e3 / ms_step,
            "ray_component_steps_per_s": n_probes * n * 5 / (ms_step * 1e-3),
            "achieved_gbs": n_probes * n * 8 / (ms_step * 1e-3) / 1e9,
            "loss_before_after_200": [l0, l1], "rel_err_f_defocus_cl": rel.tolist(),
            "plain_per_probe_path_ms_per_grad_eval": ms_plain,
            "speedup_vs_plain_per_probe": ms_plain / ms_step}


def run_only(args):
    """One workload alone (for profiler captures): W warm-up + K timed calls."""
    import torch

    import temgymcore_gb300 as t
    dev = torch.device("cuda", torch.cuda.current_device())
    if args.only in ("field-input", "field-input-astig"):
        from temgymcore_gb300.workloads import build_model, gaussian_rays, input_field
        w = input_field(seed=0, n_beams=args.beams or 16384, astigmatic=args.only == "field-input-astig")
        plan = t.FieldPlan(gaussian_rays(w["rays"]), None, grid=build_model([w["grid"]])[0])
        meth = "direct" if args.only == "field-input-astig" else "separable"
        fn = lambda: plan.evaluate(meth)  # noqa: E731
    elif args.only.startswith("field"):
        from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
        beams = args.beams or 16384
        w = beamlet_field(seed=0, n_beams=beams, astigmatic=args.only == "field-astig")
        plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
        meth = {"field-separable": "separable", "field-direct": "direct", "field-astig": "direct",
                "field-fp64": "fp64"}[args.only]
        fn = lambda: plan.evaluate(meth)  # noqa: E731
    elif args.only in ("fit", "fit-step"):
        from temgymcore_gb300.fit import StemFit
        from temgymcore_gb300.workloads import stem_fit
        w = stem_fit(seed=0)
        fit = StemFit(t.Ray(x=w["x"], y=w["y"], dx=w["dx"], dy=w["dy"], z=0.0, pathlength=0.0),
                      w["rows"], w["cols"], w["gap"], w["theta0"])
        fit.set_targets(w["theta_true"])
        fn = fit.loss_grad if args.only == "fit" else fit.step
    elif args.only == "batched":
        from temgymcore_gb300.batched import BatchedTrace
        from temgymcore_gb300.workloads import batched_sweep, build_model
        w = batched_sweep(seed=0, n_models=args.models or 512)
        bt = BatchedTrace([build_model(s) for s in w["specs"]], w["counts"], tile_rays=16384)
        bt.block, bt.rpt = 256, 2
        x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=dev) for k in ("x", "y", "dx", "dy", "tx", "ty"))
        out, raw = bt.alloc_outputs(), bt.alloc_raw()
        fn = lambda: bt.run(x, y, dx, dy, out, (tx, ty), raw)  # noqa: E731
    elif args.only == "plain":
        from temgymcore_gb300.workloads import build_model, plain_trace
        w = plain_trace(seed=0, n=args.rays or 65536)
        model = build_model(w["model"])
        ray = t.Ray(x=torch.tensor(w["x"], device=dev), y=torch.tensor(w["y"], device=dev),
                    dx=torch.tensor(w["dx"], device=dev), dy=torch.tensor(w["dy"], device=dev),
                    z=0.0, pathlength=0.0)
        acc = torch.zeros((256, 256), dtype=torch.int64, device=dev)
        fn = lambda: t.trace_to_image(ray, model, acc=acc)  # noqa: E731
    elif args.only == "transfer":
        rng = np.random.default_rng(0)
        n, m = args.rays or (1 << 20), 16
        rays = torch.tensor(np.hstack([rng.normal(0, 1e-3, (n, 4)), np.ones((n, 1))]), device=dev)
        mats = rng.normal(0, 1, (m, 5, 5))
        fn = lambda: t.transfer_rays(rays, mats)  # noqa: E731
    elif args.only in ("trace-forward", "trace-image", "trace-image-global", "trace-adjoint"):
        calls = _trace_large_calls(torch, dev, args.rays or (1 << 24))
        fn = calls[{"trace-forward": "forward", "trace-image": "forward_pixels_histogram",
                    "trace-image-global": "forward_pixels_histogram_global_atomics",
                    "trace-adjoint": "adjoint"}[args.only]]
    else:
        raise SystemExit(f"unknown --only {args.only}")
    for _ in range(args.warmup):
        fn()
    ms = _time(torch, fn, args.steps)
    print(json.dumps({"only": args.only, "ms_per_call": ms, "steps": args.steps,
                      "error_word": t._native.error_word()}))


def secondary_batched(torch, dev, hbm):
    """Batched sweep: 512 models (U{2..12} components), ~2.4e7 rays, forward +
    adjoint in one persistent launch replayed as a CUDA graph (autotuned launch
    shape), versus per-model plain launches on the same GPU."""
    import ctypes as C

    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.run import _rays_struct
    from temgymcore_gb300.workloads import batched_sweep, build_model
    w = batched_sweep(seed=0)
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"])
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=dev) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out = bt.alloc_outputs()
    raw = bt.alloc_raw()
    best, results = bt.autotune(x, y, dx, dy, out, (tx, ty), raw)
    g = bt.capture(x, y, dx, dy, out, (tx, ty), raw)
    ms = _time(torch, g.replay, 10)
    steps = int(sum(c * len(m) for c, m in zip(w["counts"], models)))
    total = int(w["counts"].sum())
    alg = total * (16 + 24 + 8)
    # per-model plain launches: forward, residual, generic adjoint per model
    packed = bt._packed
    outs = bt.alloc_outputs()
    gxy = [torch.empty(total, dtype=torch.float32, device=dev) for _ in range(2)]
    zeros = torch.zeros(total, dtype=torch.float32, device=dev)
    ws = torch.empty(64 << 20, dtype=torch.uint8, device=dev)
    raws = [torch.zeros((2 * len(m), 4), dtype=torch.float64, device=dev) for m in models]
    lib = N.lib()
    structs = []
    for m in range(len(models)):
        a, b = int(bt.offsets[m]), int(bt.offsets[m + 1])
        n = b - a
        rin = _rays_struct(n, x[a:b], y[a:b], dx[a:b], dy[a:b], None, 0.0, None, 0.0)
        rout = _rays_struct(n, outs[0][a:b], outs[1][a:b], outs[2][a:b], outs[3][a:b], None, 0.0,
                            outs[4][a:b], 0.0)
        gout = _rays_struct(n, gxy[0][a:b], gxy[1][a:b], zeros[a:b], zeros[a:b], None, 0.0, None, 0.0)
        structs.append((a, b, rin, rout, gout))

    def plain():
        for m, (a, b, rin, rout, gout) in enumerate(structs):
            mm = packed[m][0]
            lib.tg_trace_fwd(C.byref(mm), C.byref(rin), C.byref(rout), None, None, None, None, None, 0,
                             N.stream_ptr())
            torch.sub(outs[0][a:b], tx[a:b], out=gxy[0][a:b]).mul_(2.0)
            torch.sub(outs[1][a:b], ty[a:b], out=gxy[1][a:b]).mul_(2.0)
            lib.tg_trace_vjp(C.byref(mm), C.byref(rin), C.byref(gout), None, raws[m].data_ptr(),
                             ws.data_ptr(), ws.numel(), N.stream_ptr())
    ms_plain = _time(torch, plain, 2)
    return {"workload": f"batched sweep: {len(models)} models, U{{2..12}} components, {total} rays, "
                        "forward + adjoint (squared-residual loss)",
            "ms": ms, "ray_component_steps_per_s": steps / (ms * 1e-3), "rays_per_s": total / (ms * 1e-3),
            "algorithmic_bytes": alg, "achieved_gbs": alg / (ms * 1e-3) / 1e9,
            "frac_of_hbm": alg / (ms * 1e-3) / 1e9 / hbm,
            # separate forward and adjoint passes would move 64 B/ray (forward
            # 16 in + 24 out, adjoint 16 in + 8 targets); the fused launch reads
            # the inputs once, 48 B/ray
            "bytes_separate_passes": total * 64,
            "frac_of_hbm_separate_passes": total * 64 / (ms * 1e-3) / 1e9 / hbm,
            "autotuned": {"tile_rays": best[0], "block": best[1], "rays_per_thread": best[2]},
            "autotune_ms": None if results is None else [[r[1], r[2], r[3], r[0]] for r in results],
            "plain_per_model_ms": ms_plain, "speedup_vs_plain_per_model": ms_plain / ms}


def _trace_large_calls(torch, dev, n):
    """The fused chain (Lens + Detector 256x256) on n rays through the C ABI on
    device buffers: callables for the forward with pathlength, the forward +
    pixels + int64 histogram (shared-memory histograms when the workspace
    query allows, and the global-atomic path), and the adjoint with input
    gradients and per-step sums.  The returned dict keeps the buffers alive."""
    import ctypes as C

    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.run import _rays_struct, pack_model
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(0)
    x, y = (torch.tensor(rng.uniform(-1e-3, 1e-3, n).astype(np.float32), device=dev) for _ in range(2))
    dx, dy = (torch.tensor(rng.normal(0, 1e-3, n).astype(np.float32), device=dev) for _ in range(2))
    model = build_model([{"kind": "lens", "z": 0.5, "focal_length": 0.2},
                         {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (256, 256)}])
    m, keep = pack_model(model)
    o = [torch.empty(n, device=dev) for _ in range(4)]
    opl = torch.empty(n, dtype=torch.float64, device=dev)
    rin = _rays_struct(n, x, y, dx, dy, None, 0.0, None, 0.0)
    rout = _rays_struct(n, *o, None, 0.0, opl, 0.0)
    grid = model[-1]._tg_grid()
    py, px = (torch.empty(n, dtype=torch.int32, device=dev) for _ in range(2))
    hist = torch.zeros((256, 256), dtype=torch.int64, device=dev)
    g = [torch.randn(n, device=dev) for _ in range(4)]
    gi = [torch.empty(n, device=dev) for _ in range(4)]
    gout = _rays_struct(n, *g, None, 0.0, None, 0.0)
    gin = _rays_struct(n, *gi, None, 0.0, None, 0.0)
    raw = torch.zeros((4, 4), dtype=torch.float64, device=dev)
    lib = N.lib()
    ws = torch.empty(lib.tg_trace_vjp_workspace(n, C.byref(m)) + 256, dtype=torch.uint8, device=dev)
    ws_bytes = lib.tg_trace_image_workspace(n, C.byref(grid))
    hws = torch.empty(max(ws_bytes, 16), dtype=torch.uint8, device=dev)
    sp = N.stream_ptr()
    return {
        "forward": lambda: lib.tg_trace_fwd(C.byref(m), C.byref(rin), C.byref(rout), None, None, None, None,
                                            None, 0, sp),
        "forward_pixels_histogram": lambda: lib.tg_trace_image(
            C.byref(m), C.byref(rin), C.byref(rout), None, C.byref(grid), py.data_ptr(), px.data_ptr(),
            hist.data_ptr(), 1, hws.data_ptr(), ws_bytes, sp),
        "forward_pixels_histogram_global_atomics": lambda: lib.tg_trace_fwd(
            C.byref(m), C.byref(rin), C.byref(rout), None, C.byref(grid), py.data_ptr(), px.data_ptr(),
            hist.data_ptr(), 1, sp),
        "adjoint": lambda: lib.tg_trace_vjp(C.byref(m), C.byref(rin), C.byref(gout), C.byref(gin),
                                            raw.data_ptr(), ws.data_ptr(), ws.numel(), sp),
        "_shared_hist": ws_bytes > 0,
        "_keep": (keep, x, y, dx, dy, o, opl, py, px, hist, g, gi, raw, ws, hws, rin, rout, gout, gin, grid),
    }


def secondary_trace_large(torch, dev, hbm):
    """The fused chain at 16,777,216 rays (Lens + Detector): forward with
    pathlength (40 B/ray), forward + pixels + int64 histogram (48 B/ray; per-SM
    shared-memory histograms, and the global-atomic path beside it), and the
    adjoint with input gradients and per-step sums (48 B/ray), through the C
    ABI on device buffers."""
    n = 1 << 24
    calls = _trace_large_calls(torch, dev, n)
    res = {"workload": "fused chain, 16,777,216 rays, Lens + Detector 256x256",
           "histogram_path": ("per-SM shared-memory histograms (tg_trace_image)" if calls["_shared_hist"] else
                              "global atomics")}
    for name, bpr in (("forward", 40), ("forward_pixels_histogram", 48),
                      ("forward_pixels_histogram_global_atomics", 48), ("adjoint", 48)):
        ms = _time(torch, calls[name], 20)
        res[name] = {"ms": ms, "rays_per_s": n / (ms * 1e-3), "bytes_per_ray": bpr,
                     "achieved_gbs": n * bpr / (ms * 1e-3) / 1e9, "frac_of_hbm": n * bpr / (ms * 1e-3) / 1e9 / hbm}
    return res


def secondary_transfer(torch, dev, hbm):
    """transfer_rays: 1,048,576 rays through the cumulative products of 16
    transfer matrices -> (N, 16, 5) float64 (671 MB written)."""
    import temgymcore_gb300 as t
    rng = np.random.default_rng(0)
    n, m = 1 << 20, 16
    rays = torch.tensor(np.hstack([rng.normal(0, 1e-3, (n, 4)), np.ones((n, 1))]), device=dev)
    mats = rng.normal(0, 1, (m, 5, 5))
    ms = _time(torch, lambda: t.transfer_rays(rays, mats), 20)
    out_bytes = n * m * 5 * 8
    return {"workload": "transfer_rays: 1,048,576 rays x 16 cumulative 5x5 matrices, float64",
            "ms": ms, "ray_planes_per_s": n * m / (ms * 1e-3),
            "achieved_gbs": (out_bytes + n * 40) / (ms * 1e-3) / 1e9,
            "frac_of_hbm": (out_bytes + n * 40) / (ms * 1e-3) / 1e9 / hbm,
            "fp64_tflops": n * m * 50 / (ms * 1e-3) / 1e12,
            "note": "25 float64 FMAs per (ray, plane): float64-pipe bound on GB300"}


def secondary_aberrated_scan(torch, dev, hbm):
    """The headline 4D-STEM scan with an AberratedLensKrivanek (f = 0.05 m at
    z = 0.03 m; C10 = 0.02, C12 = 0.05 at 30 deg, C23 = 5 at 10 deg,
    C30 = 300 m) between the sample and the detector: the nonlinear lens
    runs inside the same fused scan kernel."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_model
    w = _workload()
    model = stem_model(w)
    kc = t.KrivanekCoeffs(C10=0.02, C12=0.05, phi12=np.deg2rad(30.0), C23=5.0, phi23=np.deg2rad(10.0),
                          C30=300.0)
    model.insert(4, t.AberratedLensKrivanek(z=0.03, focal_length=0.05, coeffs=kc))
    ray = t.Ray(x=torch.tensor(w["x"], device=dev), y=torch.tensor(w["y"], device=dev),
                dx=torch.tensor(w["dx"], device=dev), dy=torch.tensor(w["dy"], device=dev),
                z=0.0, pathlength=0.0)
    n_probes = SCAN[0] * SCAN[1]
    out = torch.empty((n_probes, 256, 256), dtype=torch.int32, device=dev)
    ms = _time(torch, lambda: t.scan_images(ray, model, out=out), 200)
    alg = n_probes * 256 * 256 * 4
    return {"workload": "4D-STEM 64x64 x 1024 rays with an aberrated lens (6 components)",
            "ms": ms, "ray_component_steps_per_s": n_probes * RAYS * (N_COMPONENTS + 1) / (ms * 1e-3),
            "achieved_gbs": alg / (ms * 1e-3) / 1e9, "frac_of_hbm": alg / (ms * 1e-3) / 1e9 / hbm,
            "hits": int(out.sum().item())}


def run_gpu(args, world, rank, local):
    import torch

    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_model
    dev = torch.device("cuda", torch.cuda.current_device())
    w = _workload()
    model = stem_model(w)
    ray = t.Ray(x=torch.tensor(w["x"], device=dev), y=torch.tensor(w["y"], device=dev),
                dx=torch.tensor(w["dx"], device=dev), dy=torch.tensor(w["dy"], device=dev),
                z=0.0, pathlength=0.0)
    n_probes = SCAN[0] * SCAN[1]
    out = torch.empty((n_probes, 256, 256), dtype=torch.int32, device=dev)
    for _ in range(args.warmup):
        t.scan_images(ray, model, out=out)
    torch.cuda.synchronize()
    a, b = _events(torch)
    _barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        a.record()
        for _ in range(args.steps):
            t.scan_images(ray, model, out=out)
        b.record()
        torch.cuda.synchronize()
    _barrier(world)
    ms = a.elapsed_time(b) / args.steps
    ms = _max_over_ranks(ms, world)
    units = n_probes * RAYS * N_COMPONENTS
    value = world * units / (ms * 1e-3)
    err = t._native.error_word()

    hbm, bf16, peak_src = _peaks()
    alg_bytes = n_probes * 256 * 256 * 4 + RAYS * 16
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    roof = {"kernel": "k_scan_hist", "bound": "hbm", "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_src,
            "algorithmic_bytes_per_launch": alg_bytes, "traffic": _traffic("k_scan_hist")}
    if args.headline_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                              "scan": list(SCAN), "roofline": roof, "clocks": clk.summary(),
                              "error_word": err}))
        return

    # end to end through the public API with host buffers
    pin_in = torch.empty((4, RAYS), dtype=torch.float32).pin_memory()
    for i, k in enumerate(("x", "y", "dx", "dy")):
        pin_in[i] = torch.from_numpy(w[k])
    pin_out = torch.empty((n_probes, 256, 256), dtype=torch.int32).pin_memory()
    dev_in = torch.empty((4, RAYS), dtype=torch.float32, device=dev)
    e2e_steps = max(3, min(args.steps, 20))

    def e2e_step():
        # ray bundle host -> device; the images go device -> host inside the
        # kernel: scan_images writes them straight into the pinned host
        # buffer across the host link (the link, ~193 GB/s, bounds this)
        dev_in.copy_(pin_in, non_blocking=True)
        r = t.Ray(x=dev_in[0], y=dev_in[1], dx=dev_in[2], dy=dev_in[3], z=0.0, pathlength=0.0)
        t.scan_images(r, model, out=pin_out)
    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    _barrier(world)
    a2, b2 = _events(torch)
    a2.record()
    for _ in range(e2e_steps):
        e2e_step()
    b2.record()
    torch.cuda.synchronize()
    e2e_ms = _max_over_ranks(a2.elapsed_time(b2) / e2e_steps, world)
    e2e = {"value": world * units / (e2e_ms * 1e-3), "unit": UNIT,
           "h2d_bytes_per_step": int(pin_in.numel() * 4), "d2h_bytes_per_step": int(pin_out.numel() * 4),
           "ms_per_step": e2e_ms, "steps": e2e_steps}
    del pin_out

    secondary = {}
    if rank == 0:
        try:
            secondary["plain_trace"] = secondary_plain(torch, dev)
        except Exception as e:  # report, never hide
            secondary["plain_trace"] = {"error": repr(e)}
        try:
            secondary["beamlet_field"] = secondary_field(torch, dev, hbm, bf16)
        except Exception as e:
            secondary["beamlet_field"] = {"error": repr(e)}
        try:
            secondary["input_field"] = secondary_input_field(torch, dev, bf16)
        except Exception as e:
            secondary["input_field"] = {"error": repr(e)}
        try:
            secondary["trace_large"] = secondary_trace_large(torch, dev, hbm)
        except Exception as e:
            secondary["trace_large"] = {"error": repr(e)}
        try:
            secondary["transfer_rays"] = secondary_transfer(torch, dev, hbm)
        except Exception as e:
            secondary["transfer_rays"] = {"error": repr(e)}
        try:
            secondary["aberrated_scan"] = secondary_aberrated_scan(torch, dev, hbm)
        except Exception as e:
            secondary["aberrated_scan"] = {"error": repr(e)}
        try:
            secondary["adjoint_fit"] = secondary_fit(torch, dev)
        except Exception as e:
            secondary["adjoint_fit"] = {"error": repr(e)}
        try:
            secondary["batched_sweep"] = secondary_batched(torch, dev, hbm)
        except Exception as e:
            secondary["batched_sweep"] = {"error": repr(e)}
    cpu = cpu_baseline() if (rank == 0 and world == 1) else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 rays / f64 binning ties", "data": "synthetic (seeded)",
            "config": headline_config(world),
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps,
            "clocks": clk.summary(), "error_word": err, "secondary": secondary}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scan", type=int, nargs=2, default=None, metavar=("ROWS", "COLS"),
                    help="smaller scan for profiling captures (default 64 64)")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the secondary workloads, e2e and CPU baseline")
    ap.add_argument("--only", default=None,
                    help="profile one workload alone: field-separable, field-direct, field-astig, "
                         "field-fp64, field-input, field-input-astig, fit, fit-step, batched, plain, "
                         "trace-forward, trace-image, trace-image-global, trace-adjoint, transfer (--rays N)")
    ap.add_argument("--beams", type=int, default=None)
    ap.add_argument("--rays", type=int, default=None)
    ap.add_argument("--models", type=int, default=None)
    args = ap.parse_args()
    if args.scan:
        global SCAN
        SCAN = tuple(args.scan)
    world, rank, local = _setup_dist(args)
    if args.only:
        run_only(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
