"""Benchmark of the GB300 TemGymCore hot path.

Headline workload (one step): the batched sweep - 512 independent optical
models with U{2..12} components drawn from lens / deflector / biprism /
aperture (log-uniform f in [0.01, 1] m), log-uniform ray counts in
[1e3, 2.6e5] (23,544,821 rays), forward trace + adjoint of the
squared-residual detector loss (the batched form of jax.value_and_grad over
run_to_end), one persistent launch replayed as a CUDA graph.  Metric:
ray-component steps per second (sum over models of rays x components),
whole job.  The working set (565 MB of inputs and targets, 1.15 GB moved per
step) exceeds the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs its own sweep (weak scaling: models
are independent, there is no data-path collective); rank 0 prints the line.
``--impl reference`` times the CPU arm: the reference's JAX path when it
imports (jax + temgym_core), else the NumPy float64 restatement of its
per-model value-and-gradient, over the whole sweep on all host cores.
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

METRIC = "fwd+grad ray\u00b7component steps/s; field beam\u00b7px/s at stated err vs FP64 oracle"
UNIT = "ray\u00b7component steps/s"
SWEEP_SEED = 0
SWEEP_MODELS = 512
# bytes per ray of the fused forward + adjoint launch: x, y, dx, dy and the
# two targets read (24), x, y, dx, dy written (16), pathlength (8), alive (1)
SWEEP_BYTES_PER_RAY = 49
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


def _fp32_roofline(torch, ms, pairs):
    """The fast direct field against the FP32 issue rate: the strip recurrence
    costs 10 FP32 instructions per (beam, pixel) (z <- z w and w <- w rho: two
    FMUL + two FFMA each; two FADD into the sums); the peak is 128 FP32 lanes
    per SM at the measured maximum SM clock."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            mhz, src = float(json.load(fh)["sm_max_mhz"]), "measured max SM clock"
    except Exception:
        mhz, src = 2070.0, "nominal max SM clock"
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    achieved = 10 * pairs / (ms * 1e-3) / 1e12
    peak = sms * 128 * mhz * 1e6 / 1e12
    return {"bound": "fp32", "instr_per_beam_px": 10, "achieved": achieved, "peak": peak,
            "unit": "T FP32 lane-instructions/s", "frac": achieved / peak,
            "peak_source": f"{sms} SMs x 128 FP32 lanes x {mhz:.0f} MHz ({src})"}


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


_SWEEP = {}


def _sweep():
    """The headline workload's seeded inputs (cached per process)."""
    if not _SWEEP:
        from temgymcore_gb300.workloads import batched_sweep
        w = batched_sweep(seed=SWEEP_SEED, n_models=SWEEP_MODELS)
        w["offsets"] = np.concatenate([[0], np.cumsum(w["counts"])])
        w["work"] = np.array([int(c) * len(sp) for c, sp in zip(w["counts"], w["specs"])], dtype=np.int64)
        _SWEEP.update(w)
    return _SWEEP


def headline_config(world: int) -> dict:
    """The headline workload (both arms print this config)."""
    w = _sweep()
    return {"workload": "batched sweep: 512 models, U{2..12} components from lens/deflector/biprism/"
                        "aperture (log-uniform f in [0.01, 1] m), log-uniform rays per model in "
                        "[1e3, 2.6e5], forward + adjoint of the squared-residual detector loss "
                        "(per-model loss and per-step gradient sums), seed 0",
            "models": len(w["specs"]), "rays_per_step": int(w["offsets"][-1]),
            "ray_component_steps_per_step": int(w["work"].sum()),
            "l2": "no flush: 565 MB of inputs and targets read, 590 MB written per step > 129 MB L2",
            "parallelism": f"dp{world} (independent sweeps per rank)"}


# ------------------------------------------------------------ CPU baselines

def _cpu_sweep_chunk(models):
    """The oracle's float64 value-and-gradient (forward with its tape, loss,
    reverse walk: what jax.value_and_grad over run_to_end does) for the given
    sweep models.  Returns (seconds, ray-component steps)."""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from oracle.adjoint import value_and_raw
    w = _sweep()
    off = w["offsets"]
    t0 = time.perf_counter()
    steps = 0
    for m in models:
        a, b = int(off[m]), int(off[m + 1])
        value_and_raw(w["specs"][m], *(w[k][a:b].astype(np.float64) for k in ("x", "y", "dx", "dy", "tx", "ty")))
        steps += int(w["work"][m])
    return time.perf_counter() - t0, steps


def cpu_baseline():
    """Single-thread oracle value-and-gradient over the whole sweep (rank 0, N=1)."""
    el, steps = _cpu_sweep_chunk(list(range(len(_sweep()["specs"]))))
    return {"value": steps / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "the whole 512-model sweep once (all 23,544,821 rays): NumPy float64 restatement "
                      "of run_to_end + squared-residual loss + reverse-mode gradient per model, 1 thread",
            "seconds": el}


def _jax_probe():
    """Whether the reference's own JAX path imports here (the driver's
    baseline/_ref install first on the path)."""
    ref = os.path.join(ROOT, "baseline", "_ref")
    if os.path.isdir(ref) and ref not in sys.path:
        sys.path.insert(0, ref)
    try:
        import jax  # noqa: F401
        import temgym_core  # noqa: F401
    except Exception as e:  # the normal case: jax is not installed on this image
        return f"unavailable: {type(e).__name__}: {e}"
    return ("jax and temgym_core import, but the reference has no Aperture component, so it "
            "cannot express this workload; the timed arm is the NumPy restatement")


def _windows(work, target, n_workers, n_windows):
    """Per step: a window of models (cycling through a fixed shuffled order)
    holding about ``target`` ray-component steps, dealt to the workers
    heaviest first onto the least-loaded worker."""
    order = np.random.default_rng(0).permutation(len(work))
    pos, out = 0, []
    for _ in range(n_windows):
        take, acc = [], 0
        while acc < target and len(take) < len(work):
            m = int(order[pos % len(order)])
            take.append(m)
            acc += int(work[m])
            pos += 1
        chunks, load = [[] for _ in range(n_workers)], [0] * n_workers
        for m in sorted(take, key=lambda m: -int(work[m])):
            i = load.index(min(load))
            chunks[i].append(m)
            load[i] += int(work[m])
        out.append([c for c in chunks if c])
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    jax_state = _jax_probe()
    w = _sweep()
    total = int(w["work"].sum())
    # size each step so the whole --steps/--warmup run stays near 90 s
    t, n = _cpu_sweep_chunk(list(range(8)))
    rate = n / max(t, 1e-9) * cores
    target = int(min(total, max(1, 90.0 / (args.steps + args.warmup) * rate)))
    wins = _windows(w["work"], target, cores, args.steps + args.warmup)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_sweep) as pool:
        def step(chunks):
            t0 = time.perf_counter()
            r = pool.map(_cpu_sweep_chunk, chunks)
            return time.perf_counter() - t0, sum(x[1] for x in r)
        for i in range(args.warmup):
            step(wins[i])
        res = [step(wins[args.warmup + i]) for i in range(args.steps)]
    secs = sum(r[0] for r in res)
    steps = sum(r[1] for r in res)
    v = steps / secs
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded), no dataset",
            "config": headline_config(1),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"per step a window of sweep models holding ~{target} of the "
                                       f"{total} ray-component steps (windows cycle through all 512 "
                                       f"models), {cores} spawn workers, NumPy float64 value-and-gradient",
                             "jax_reference": jax_state},
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
    # CPU baseline (1 thread): the oracle's run_to_end + metres_to_pixels +
    # into_image + the model's ABCD, repeated for about 3 s
    import oracle
    from oracle.rays import ORay
    g = {"pixel_size": (1e-5, 1e-5), "shape": (256, 256)}
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 3.0:
        o = oracle.run_to_end(ORay.from_f32(w["x"], w["y"], w["dx"], w["dy"], 0.0, 0.0), w["model"])
        py, px = oracle.metres_to_pixels(g, o.x, o.y)
        oracle.into_image(g, py, px)
        oracle.model_abcd(ORay(np.zeros(1), np.zeros(1), np.zeros(1), np.zeros(1), 0.0, 0.0), w["model"])
        reps += 1
    el = (time.perf_counter() - t0) / reps
    cpu = {"value": 2 * n / el, "unit": UNIT, "cores": 1, "kind": "port", "ms_per_call": 1e3 * el,
           "sample": f"the whole 65,536-ray workload, {reps} repetitions: NumPy float64 run_to_end + "
                     "metres_to_pixels + into_image + ABCD, 1 thread"}
    return {"workload": "plain trace 65,536 rays, Lens+Detector 256x256, fused trace+pixels+hist",
            "cpu_baseline": cpu,
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


def _pixel_sample(shape, n_random=4096):
    """Flat pixel indices: the central 32 x 32 block (where the diffraction
    pattern is bright) and n_random seeded random pixels."""
    h, w = shape
    yy, xx = np.meshgrid(np.arange(h // 2 - 16, h // 2 + 16), np.arange(w // 2 - 16, w // 2 + 16), indexing="ij")
    rnd = np.random.default_rng(7).choice(h * w, n_random, replace=False)
    return np.unique(np.concatenate([(yy * w + xx).ravel(), rnd]))


def _oracle_field_leg(images, oracle_fn, n_beams, idx):
    """CPU baseline of a beamlet-field workload and the error of each GPU
    image against the float64 oracle (exact k*pathlength reduction) at the
    pixel sample idx: the oracle's chunked sum over every beam at those
    pixels, 1 thread, timed."""
    t0 = time.perf_counter()
    ref = oracle_fn(idx)
    el = time.perf_counter() - t0
    scale = np.max(np.abs(ref))
    bright = np.abs(ref) > 0.25 * scale
    errs = {}
    for name, img in images.items():
        g = img.reshape(-1)[idx].astype(np.complex128)
        errs[name] = {"field_rel_err_vs_fp64_oracle": float(np.max(np.abs(g - ref)) / scale),
                      "phase_err_rad_bright_vs_fp64_oracle":
                          float(np.max(np.abs(np.angle(g[bright] * np.conj(ref[bright]))))) if bright.any() else None}
    cpu = {"value": n_beams * idx.size / el, "unit": "beam\u00b7px/s", "cores": 1, "kind": "port",
           "sample": f"all {n_beams} beams x {idx.size} pixels (the central 32x32 block and seeded random "
                     "pixels): NumPy complex128 make_gaussian_image restatement, chunks of 64 beams, 1 thread",
           "seconds": el}
    return cpu, errs


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
    import oracle.field as of
    idx = _pixel_sample((512, 512), 2048)
    cpu, errs = _oracle_field_leg({n: plan.evaluate(n).cpu().numpy() for n in ("separable", "direct")},
                                  lambda i: of.evaluate_gaussian_input_image(w["rays"], w["grid"], pixel_index=i),
                                  16384, idx)
    res["cpu_baseline"] = cpu
    res["separable_gemm"].update(errs["separable"])
    res["direct_fast"].update(errs["direct"])
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
    res["direct_fast"] = {"ms": ms_dir, "beam_px_per_s": pairs / (ms_dir * 1e-3),
                          "roofline": _fp32_roofline(torch, ms_dir, pairs)}
    res["direct_fp64"] = {"ms": ms_f64, "beam_px_per_s": pairs / (ms_f64 * 1e-3)}
    res["speedup_separable_vs_fp64"] = ms_f64 / ms_sep
    res["prep_plan_ms"] = ms_prep
    # the adjoint (tg_field_vjp_ex): gradients of sum |F - T|^2 with respect to
    # every beam's amplitude, pathlength, x, y, dx, dy and the model's steps
    T = torch.zeros(plan.shape, dtype=torch.complex64, device=dev)
    G = 2 * (plan.evaluate("separable").clone() - T)
    ms_vjp = _time(torch, lambda: plan.vjp(G, method="separable"), 10)
    ms_vjp_dir = _time(torch, lambda: plan.vjp(G, method="direct"), 3)
    res["adjoint"] = {"ms": ms_vjp, "beam_px_per_s": pairs / (ms_vjp * 1e-3),
                      "note": "separable beams: the six complex moments per beam from one split-BF16 GEMM "
                              "(conj(G) against the column factors times dc^0..2) and a pass over the rows, "
                              "then the float64 forward-mode chain rule per beam",
                      "direct_moments_ms": ms_vjp_dir}
    # errors against the all-float64 kernel's image
    ref = plan.evaluate("fp64").clone().cpu().numpy().astype(np.complex128)
    _field_errors(plan, ref, ("separable", "direct"),
                  {"separable": res["separable_gemm"], "direct": res["direct_fast"]})
    # astigmatic case (direct kernel only)
    wa = beamlet_field(seed=0, astigmatic=True)
    pa = t.FieldPlan(gaussian_rays(wa["rays"]), build_model(wa["model"]))
    ms_a = _time(torch, lambda: pa.evaluate("direct"), 3)
    res["astigmatic_direct"] = {"ms": ms_a, "beam_px_per_s": pairs / (ms_a * 1e-3), "separable": pa.separable,
                                "roofline": _fp32_roofline(torch, ms_a, pairs)}
    # CPU baseline and the errors against the float64 oracle at a pixel sample
    import oracle.field as of
    idx = _pixel_sample((512, 512))
    imgs = {n: plan.evaluate(n).cpu().numpy() for n in ("separable", "direct", "fp64")}
    cpu, errs = _oracle_field_leg(imgs, lambda i: of.make_gaussian_image(w["rays"], w["model"], pixel_index=i),
                                  16384, idx)
    res["cpu_baseline"] = cpu
    for n, e in errs.items():
        res.setdefault({"separable": "separable_gemm", "direct": "direct_fast", "fp64": "direct_fp64"}[n], {}).update(e)
    _, ea = _oracle_field_leg({"direct": pa.evaluate("direct").cpu().numpy()},
                              lambda i: of.make_gaussian_image(wa["rays"], wa["model"], pixel_index=i), 16384, idx)
    res["astigmatic_direct"].update(ea["direct"])
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
    idf, idt = fit.identifiable(), fit.identifiable(w["theta_true"])
    rel_id = np.abs(idf - idt) / np.abs(idt)
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
    cpu = _cpu_fit_step(w)
    return {"workload": "adjoint fit: 32x32 scan x 1,024 rays (1,048,576 rays), 21 parameters, "
                        "loss = sum of squared detector residuals",
            "cpu_baseline": cpu,
            "loss_grad_ms": ms_lg, "adam_step_graph_ms": ms_step,
            "grad_evals_per_s": 1e3 / ms_step,
            "ray_component_steps_per_s": n_probes * n * 6 / (ms_step * 1e-3),
            "achieved_gbs": n_probes * n * 8 / (ms_step * 1e-3) / 1e9,
            "loss_before_after_200": [l0, l1],
            "identifiable_rel_err": dict(zip(("A", "b", "K00", "K01", "K10", "K11"), rel_id.tolist())),
            "rel_err_f_defocus_cl": rel.tolist(),
            "note_identifiability": "the detector positions fix 6 combinations of the 21 parameters "
                                    "(position gain A, slope gain b = A defocus + B, 2x2 scan response K); "
                                    "f, defocus and camera length individually are not identifiable",
            "plain_per_probe_path_ms_per_grad_eval": ms_plain,
            "speedup_vs_plain_per_probe": ms_plain / ms_step}


def _cpu_fit_step(w):
    """CPU baseline of one fit step (1 thread): per probe, the oracle's
    float64 value-and-gradient of the squared detector residual (targets from
    the oracle at the perturbed parameters, formed before the clock starts);
    the chain rule from per-step sums to the 21 parameters is O(1) per probe
    and left out."""
    import oracle
    from oracle.adjoint import value_and_raw
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import stem_fit_probe_spec

    def specs(theta):
        sg, spec = stem_fit_probe_spec(w, theta, 0)
        yy, xx = np.meshgrid(np.arange(w["rows"]), np.arange(w["cols"]), indexing="ij")
        spx, spy = oracle.pixels_to_metres(sg, yy.ravel(), xx.ravel())
        out = []
        for p in range(w["rows"] * w["cols"]):
            sp = [dict(c) for c in spec]
            for c in sp:
                if c["kind"] in ("scanner", "descanner"):
                    c["scan_pos_x"], c["scan_pos_y"] = float(spx[p]), float(spy[p])
            out.append(sp)
        return out
    v = [w[k].astype(np.float64) for k in ("x", "y", "dx", "dy")]
    tgt = [oracle.run_to_end(ORay(*v, 0.0, 0.0), sp) for sp in specs(w["theta_true"])]
    s0 = specs(w["theta0"])
    t0 = time.perf_counter()
    for sp, tr in zip(s0, tgt):
        value_and_raw(sp, *v, tr.x, tr.y)
    el = time.perf_counter() - t0
    n = len(s0) * v[0].size
    return {"value": n * 6 / el, "unit": UNIT, "cores": 1, "kind": "port", "ms_per_grad_eval": 1e3 * el,
            "sample": f"one whole loss + gradient evaluation ({len(s0)} probes x {v[0].size} rays, 6 "
                      "components): NumPy float64 value-and-gradient per probe, 1 thread"}


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
    elif args.only == "field-vjp":
        from temgymcore_gb300.workloads import beamlet_field, build_model, gaussian_rays
        w = beamlet_field(seed=0, n_beams=args.beams or 16384)
        plan = t.FieldPlan(gaussian_rays(w["rays"]), build_model(w["model"]))
        G = 2 * plan.evaluate().clone()
        fn = lambda: plan.vjp(G)  # noqa: E731
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
        bt.block, bt.rpt = 512, 2
        x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=dev) for k in ("x", "y", "dx", "dy", "tx", "ty"))
        out, raw, alive, loss = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
        fn = lambda: bt.run(x, y, dx, dy, out, (tx, ty), raw, alive=alive, loss=loss)  # noqa: E731
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


def headline_setup(torch, dev):
    """The batched sweep on the device: plan, autotuned launch shape, and the
    forward + adjoint launch captured as a CUDA graph."""
    from temgymcore_gb300.batched import BatchedTrace
    from temgymcore_gb300.workloads import build_model
    w = _sweep()
    models = [build_model(s) for s in w["specs"]]
    bt = BatchedTrace(models, w["counts"], tile_rays=16384)
    x, y, dx, dy, tx, ty = (torch.tensor(w[k], device=dev) for k in ("x", "y", "dx", "dy", "tx", "ty"))
    out, raw, alive, loss = bt.alloc_outputs(), bt.alloc_raw(), bt.alloc_alive(), bt.alloc_loss()
    best, results = bt.autotune(x, y, dx, dy, out, (tx, ty), raw, alive=alive, loss=loss)
    g = bt.capture(x, y, dx, dy, out, (tx, ty), raw, alive=alive, loss=loss)
    return {"w": w, "models": models, "bt": bt, "io": (x, y, dx, dy, tx, ty), "out": out, "raw": raw,
            "alive": alive, "loss": loss, "graph": g, "best": best, "results": results}


def batched_vs_per_model(torch, dev, H, ms):
    """The plain per-model kernel path on the same GPU (per model: fused
    forward launch, the residual in torch, the generic adjoint launch) against
    the batched launch (ms per step)."""
    import ctypes as C

    from temgymcore_gb300 import _native as N
    from temgymcore_gb300.run import _rays_struct
    bt, models = H["bt"], H["models"]
    x, y, dx, dy, tx, ty = H["io"]
    total = bt.total
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
    return {"workload": "the headline sweep through per-model plain launches (forward, residual, generic "
                        "adjoint per model; apertures not applied)",
            "plain_per_model_ms": ms_plain, "batched_ms": ms,
            "speedup_batched_vs_plain_per_model": ms_plain / ms}


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
            "f64_equivalent_tflops": n * m * 50 / (ms * 1e-3) / 1e12,
            "note": "25 multiply-adds per (ray, plane) carried in double-float (float32 pairs, "
                    "k_transfer_rays_df): issue-bound on the float32 arithmetic; the float64 "
                    "kernel takes only entries outside the double-float range"}


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


def secondary_stem(torch, dev, hbm, world):
    """4D-STEM shadow images (64 x 64 scan x 1,024 rays, per-probe dense
    256 x 256 int32 images): the fused scan kernel, its roofline, the call
    through the public API with host buffers, and a 1-thread CPU baseline."""
    import temgymcore_gb300 as t
    from temgymcore_gb300.workloads import stem_model
    w = _workload()
    model = stem_model(w)
    ray = t.Ray(x=torch.tensor(w["x"], device=dev), y=torch.tensor(w["y"], device=dev),
                dx=torch.tensor(w["dx"], device=dev), dy=torch.tensor(w["dy"], device=dev),
                z=0.0, pathlength=0.0)
    n_probes = SCAN[0] * SCAN[1]
    out = torch.empty((n_probes, 256, 256), dtype=torch.int32, device=dev)
    ms = _time(torch, lambda: t.scan_images(ray, model, out=out), 200)
    units = n_probes * RAYS * N_COMPONENTS
    alg = n_probes * 256 * 256 * 4 + RAYS * 16
    res = {"workload": "4D-STEM shadow images: 64x64 scan (step 1e-9 m, rotation U(0,2pi)), 1024-ray "
                       "point-source bundle per probe, descan I+N(0,1e-3), camera length 0.1 m, 256x256 "
                       "int32 images at 5.5e-5 m",
           "ms": ms, "ray_component_steps_per_s": units / (ms * 1e-3),
           "roofline": {"kernel": "k_scan_hist", "bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9,
                        "peak": hbm, "unit": "GB/s", "frac": alg / (ms * 1e-3) / 1e9 / hbm,
                        "algorithmic_bytes_per_launch": alg, "traffic": _traffic("k_scan_hist")}}
    # through the public API with host buffers: the ray bundle host -> device,
    # the images written by the kernel straight into pinned host memory
    pin_in = torch.empty((4, RAYS), dtype=torch.float32).pin_memory()
    for i, k in enumerate(("x", "y", "dx", "dy")):
        pin_in[i] = torch.from_numpy(w[k])
    pin_out = torch.empty((n_probes, 256, 256), dtype=torch.int32).pin_memory()
    dev_in = torch.empty((4, RAYS), dtype=torch.float32, device=dev)

    def e2e_step():
        dev_in.copy_(pin_in, non_blocking=True)
        r = t.Ray(x=dev_in[0], y=dev_in[1], dx=dev_in[2], dy=dev_in[3], z=0.0, pathlength=0.0)
        t.scan_images(r, model, out=pin_out)
    e2e_ms = _time(torch, e2e_step, 10)
    res["e2e"] = {"value": units / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                  "h2d_bytes_per_step": int(pin_in.numel() * 4), "d2h_bytes_per_step": int(pin_out.numel() * 4)}
    del pin_out
    # CPU baseline (1 thread): the per-probe loop of run_to_end + into_image
    import oracle
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import stem_probe_model
    g = {k: w["detector"][k] for k in ("pixel_size", "shape")}
    sg = {k: w["scangrid"][k] for k in ("pixel_size", "shape", "rotation")}
    probes = 1024
    t0 = time.perf_counter()
    for p in range(probes):
        r, c = divmod(p, SCAN[1])
        spx, spy = oracle.pixels_to_metres(sg, r, c)
        o = oracle.run_to_end(ORay(w["x"].astype(np.float64), w["y"].astype(np.float64),
                                   w["dx"].astype(np.float64), w["dy"].astype(np.float64), 0.0, 0.0),
                              stem_probe_model(w, float(spx), float(spy)))
        py, px = oracle.metres_to_pixels(g, o.x, o.y)
        oracle.into_image(g, py, px)
    el = time.perf_counter() - t0
    res["cpu_baseline"] = {"value": probes * RAYS * N_COMPONENTS / el, "unit": UNIT, "cores": 1,
                           "kind": "port",
                           "sample": f"{probes} of {n_probes} probes x {RAYS} rays: NumPy float64 run_to_end + "
                                     "metres_to_pixels + into_image per probe, 1 thread"}
    return res


def run_gpu(args, world, rank, local):
    import torch

    import temgymcore_gb300 as t
    dev = torch.device("cuda", torch.cuda.current_device())
    hbm, bf16, peak_src = _peaks()
    H = headline_setup(torch, dev)
    bt, g = H["bt"], H["graph"]
    w = H["w"]
    units = int(w["work"].sum())
    for _ in range(args.warmup):
        g.replay()
    torch.cuda.synchronize()
    a, b = _events(torch)
    _barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        a.record()
        for _ in range(args.steps):
            g.replay()
        b.record()
        torch.cuda.synchronize()
    _barrier(world)
    ms = a.elapsed_time(b) / args.steps
    ms = _max_over_ranks(ms, world)
    value = world * units / (ms * 1e-3)
    err = t._native.error_word()
    alg_bytes = bt.total * SWEEP_BYTES_PER_RAY
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    tr = _traffic("k_batch")
    roof = {"kernel": "k_batch", "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": peak_src, "algorithmic_bytes_per_launch": alg_bytes,
            "bytes_per_ray": SWEEP_BYTES_PER_RAY, "traffic": tr,
            "timing": "graph replay of one step (the work-counter memset + k_batch) with CUDA events"}
    if args.headline_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                              "roofline": roof, "clocks": clk.summary(), "error_word": err}))
        return

    # end to end through the public API with host buffers: value_and_grad
    # copies the six input arrays in from pinned host memory and the loss and
    # per-step gradient sums back, every step
    host = [torch.from_numpy(w[k]).pin_memory() for k in ("x", "y", "dx", "dy", "tx", "ty")]
    for _ in range(2):
        bt.value_and_grad(*host)
    torch.cuda.synchronize()
    _barrier(world)
    e2e_steps = max(3, min(args.steps, 20))
    a2, b2 = _events(torch)
    a2.record()
    for _ in range(e2e_steps):
        bt.value_and_grad(*host, sync=False)
    b2.record()
    torch.cuda.synchronize()
    e2e_ms = _max_over_ranks(a2.elapsed_time(b2) / e2e_steps, world)
    e2e = {"value": world * units / (e2e_ms * 1e-3), "unit": UNIT,
           "h2d_bytes_per_step": int(sum(h.numel() * 4 for h in host)),
           "d2h_bytes_per_step": int(len(H["models"]) * 8 + int(bt.info.total_steps) * 4 * 8),
           "ms_per_step": e2e_ms, "steps": e2e_steps, "call": "BatchedTrace.value_and_grad(host tensors)"}

    secondary = {}
    if rank == 0:
        secondary["batched_autotune"] = {
            "chosen": {"tile_rays": H["best"][0], "block": H["best"][1], "rays_per_thread": H["best"][2]},
            "candidates_ms": None if H["results"] is None else [[r[1], r[2], r[3], r[0]] for r in H["results"]]}
        for name, fn in (("batched_vs_per_model", lambda: batched_vs_per_model(torch, dev, H, ms)),
                         ("stem_4d", lambda: secondary_stem(torch, dev, hbm, world)),
                         ("plain_trace", lambda: secondary_plain(torch, dev)),
                         ("beamlet_field", lambda: secondary_field(torch, dev, hbm, bf16)),
                         ("input_field", lambda: secondary_input_field(torch, dev, bf16)),
                         ("trace_large", lambda: secondary_trace_large(torch, dev, hbm)),
                         ("transfer_rays", lambda: secondary_transfer(torch, dev, hbm)),
                         ("aberrated_scan", lambda: secondary_aberrated_scan(torch, dev, hbm)),
                         ("adjoint_fit", lambda: secondary_fit(torch, dev))):
            try:
                secondary[name] = fn()
            except Exception as e:  # report, never hide
                secondary[name] = {"error": repr(e)}
    del H
    cpu = cpu_baseline() if (rank == 0 and world == 1) else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 rays / f64 composition, moments and pathlength",
            "data": "synthetic (seeded)", "config": headline_config(world),
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps,
            "clocks": clk.summary(), "error_word": err, "secondary": secondary}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scan", type=int, nargs=2, default=None, metavar=("ROWS", "COLS"),
                    help="smaller scan for profiling captures (default 64 64)")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the secondary workloads, e2e and CPU baseline")
    ap.add_argument("--only", default=None,
                    help="profile one workload alone: field-separable, field-direct, field-astig, field-vjp, "
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
