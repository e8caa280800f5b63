#!/usr/bin/env python
"""Benchmark: inpainted Mpix/s of the multiscale non-local inpainting path.

A step is one ImageInpainting::process of the 512x512 nlpoisson workload
(Voronoi texture, 6-ellipse hole of ~15%, L2Combined, lambda 0.05, patch 9,
scales 8, coarse 0.1, CG tolerance 1e-4, seeded synthetic input).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value`: Mpix/s with the input already in HBM (nli_process_device), timed
with CUDA events on the launching stream; L2 (129 MB) is flushed with a
256 MB write between timed steps.  `e2e`: the same through nli_process with
pinned host buffers (host->device input copy and device->host result copy
inside the timed region).  N > 1 runs independent replicas, one per GPU
(the path has no exchange step), weak scaling.

The reference arm (--impl reference) times the reference algorithm on the
host cores: the CPU restatement of the reference (oracle/, bit-identical to
the reference's serial build; its PatchMatch is the reference's OpenMP
variant) on a bounded sample per step -- one PatchMatch and one update on
every pyramid scale -- scaled to a whole process() by the reference's own
per-scale iteration counts of this workload.
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

import __graft_entry__ as ge  # noqa: E402

METRIC = "inpainted Mpix/s on 1 GB300, batched vs plain GPU path, ≤0.1 dB PSNR gap to ref"
UNIT = "Mpix/s"
# algorithmic FP32 work of one patch distance, P = 9: 31 P^2 + 8 (C = 3,
# L2Combined: 9 differences, 9 squares/FMAs and 2 weighted FMAs per tap);
# 44 P^2 + 8 for the 4-channel L2 RGBD distance
FLOP_PER_CANDIDATE = 31 * 81 + 8
FLOP_PER_CANDIDATE_RGBD = 44 * 81 + 8
# the workload of the run (--workload); the headline is the 512x512 NL-Poisson one
WORKLOAD = "nlpoisson512"
WORKLOADS = {
    "nlpoisson512": ("512x512 RGB float32 Voronoi (40 seeds) + oriented sinusoids, union of 6 ellipses (~15% hole); "
                     "nlpoisson + L2Combined, lambda 0.05, psigma 10000, patch 9, scales 8, coarse 0.1, CG tol 1e-4, "
                     "iters 200, tol 0.1, conft 5, confa 0.1, init poisson, PatchMatch 10 sweeps / 30 shots"),
    "nlmeans256": ("256x256 RGB float32 smooth gradient + stripes (period 12) + noise (sigma 3), centred disc of "
                   "radius 32 (~4.9% hole); nlmeans + L2Combined, lambda 0.05, psigma 10000, patch 9, scales 5, "
                   "coarse 0.1, iters 200, tol 0.1, conft 5, confa 0.1, init poisson, PatchMatch 10 sweeps / 30 shots"),
    "nldepth640": ("640x480 RGB-D float32 Voronoi (60 seeds) + depth of 3-8 planes in [0.5, 5] m, 10 brush strokes "
                   "(~12% hole); nldepth + L2RGBD, lambda_rgb 1.0, lambda_d 0.0, psigma 10000, patch 9, scales 9, "
                   "coarse 0.1, iters 200, tol 0.1, conft 5, confa 0.1, init poisson, PatchMatch 10 sweeps / 30 shots"),
}
# algorithmic bytes of one CG iteration per unknown and channel: read d, a1,
# a2-links, x, r, q; write x, r, d (float32), as counted for the roofline
CG_BYTES_PER_UNKNOWN_ITER = 32
L2_FLUSH_BYTES = 256 << 20
COUNTS = os.path.join(ROOT, "tests", "golden", "config2_reference_counts.json")
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# ncu summary of the dominant kernel; its "traffic_bytes_per_launch:" line is
# the DRAM bytes (read + write) of one finest-scale sweep
TRAFFIC = os.path.join(ROOT, "profiles", "pm_sweep_l2combined_512x512.md")
# the CPU baseline's build of the reference algorithm (oracle/build.py)
TIMING_FLAGS = "g++ -O3 -DNDEBUG -std=gnu++17 -fopenmp (the reference's Release build flags)"
GOLDEN = os.path.join(ROOT, "tests", "golden")


def workload_desc():
    return WORKLOADS[WORKLOAD]


def workload(seed=0):
    ge.package()
    from nli_gb300 import workloads as wl
    if WORKLOAD == "nlmeans256":
        return wl.config1(seed=seed)
    if WORKLOAD == "nldepth640":
        return wl.config3(seed=seed)
    return wl.config2(seed=seed)


def flop_per_candidate():
    return FLOP_PER_CANDIDATE_RGBD if WORKLOAD == "nldepth640" else FLOP_PER_CANDIDATE


class Clocks:
    """nvidia-smi samples (every 200 ms) while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out = self.proc.communicate(timeout=5)[0]
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out = self.proc.communicate()[0]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def reference_counts():
    """Per-scale PatchMatch / update call counts of the reference on this
    workload (serial run, committed fixture), finest scale first; the
    fixture covers the 512x512 NL-Poisson workload."""
    if WORKLOAD == "nlpoisson512" and os.path.exists(COUNTS):
        with open(COUNTS) as f:
            c = json.load(f)
        return c["iterations"], "reference run (seed %d)" % c.get("seed", 0)
    return None, None


def cpu_sample(img, mask, p, iterations):
    """Times one PatchMatch (OpenMP, all host threads) and one update on
    every scale with the oracle restatement and returns (estimated seconds
    of a whole process(), wall seconds spent, threads)."""
    from oracle import oracle as O
    orc = O.Oracle(timing=True)
    S = p.scales
    imgs, masks = [np.asarray(img, np.float32)], [np.asarray(mask, np.uint8)]
    for i in range(1, S):
        a, b = orc.downsample_with_mask(imgs[-1], masks[-1], p.subsampling_rate, 0.4, False)
        imgs.append(a)
        masks.append(b)
    t_pm, t_up = [], []
    wall0 = time.perf_counter()
    for lvl in range(S):
        im = orc.poisson_init(imgs[lvl], masks[lvl])
        ext = orc.extended_domain(masks[lvl], p.update.patch_x, p.update.patch_y)
        src, tgt, _ = orc.scale_masks(ext, p.update.patch_x // 2, True)
        conf = orc.confidence_mask(masks[lvl], p.conf_decay_time, p.conf_asymptotic)
        t0 = time.perf_counter()
        nnf = orc.patchmatch(p.distance, p.patchmatch, im, src, im, tgt, seed=lvl, parallel=True)[0]
        t1 = time.perf_counter()
        orc.update(p.update, im, im, masks[lvl], ext, nnf, conf)
        t2 = time.perf_counter()
        t_pm.append(t1 - t0)
        t_up.append(t2 - t1)
    wall = time.perf_counter() - wall0
    est = 0.0
    for lvl in range(S):
        est += iterations[lvl] * (t_pm[lvl] + t_up[lvl])
        if lvl < S - 1:  # propagate_weights into this scale: 2 PatchMatch + 1 update
            est += t_pm[lvl + 1] + t_pm[lvl] + t_up[lvl]
    return est, wall, orc.max_threads


def formula_candidates(st, pm_iterations=10):
    """The candidates the reference's PatchMatch evaluates in one process()
    by the hot-path formula: per call N_t (1 + I (2 + W_rs)), with N_t the
    scale's target points, I the sweeps and W_rs = floor(log2 max(W, H)) + 1
    random-search windows; calls per scale = its iterations plus one per
    scale transition it takes part in (propagate_weights runs PatchMatch on
    the coarser and on the finer scale)."""
    import math
    S = st["scales"]
    total = 0
    for l in range(S):
        W, H, nt = st["width"][l], st["height"][l], st["targets"][l]
        windows = int(math.floor(math.log2(max(W, H)))) + 1
        calls = st["iterations"][l] + (1 if l < S - 1 else 0) + (1 if l > 0 else 0)
        total += calls * nt * (1 + pm_iterations * (2 + windows))
    return total


def cpu_calibration():
    """Checks the per-scale sampling of cpu_sample against a whole timed
    process() on the 256x256 NL-means workload: the OpenMP restatement (the
    reference's Release flags) runs the whole process() once, then the
    sampled estimate is formed with that run's own per-scale iteration
    counts.  Returns {measured_s, estimated_s, ratio, ...}."""
    from oracle import oracle as O
    from nli_gb300 import workloads as wl
    orc = O.Oracle(timing=True)
    img, mask, p = wl.config1(seed=0)
    orc.process(img[:64, :64].copy(), mask[:64, :64].copy(), p, parallel=True)  # warm the threads
    t0 = time.perf_counter()
    _, st = orc.process(img, mask, p, seed=101, parallel=True, return_stats=True)
    measured = time.perf_counter() - t0
    est, wall, threads = cpu_sample(img, mask, p, list(st["iterations"][:p.scales]))
    return {"workload": "256x256 NL-means (nlmeans256), one whole OpenMP process()", "measured_s": measured,
            "estimated_s": est, "ratio": est / measured, "sample_wall_s": wall, "cores": threads,
            "iterations": list(st["iterations"][:p.scales])}


def max_over_ranks(value, device="cpu"):
    """The largest `value` over the ranks of the default process group (the
    value itself with one rank): the job's time is its slowest rank's."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, steps, mpix_per_rank_step, total_ms):
    """Whole-job Mpix/s: every rank processes its own images (replicas), so
    the units of all ranks divide the slowest rank's time."""
    return world * steps * mpix_per_rank_step / (total_ms / 1e3)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    img, mask, p = workload()
    iters, source = reference_counts()
    if iters is None:
        print(json.dumps({"impl": "reference", "unavailable": "per-scale iteration counts of the reference run "
                          "(tests/golden/config2_reference_counts.json) are missing"}))
        return 0
    mpix = img.shape[0] * img.shape[1] / 1e6
    for _ in range(args.warmup):
        cpu_sample(img, mask, p, iters)
    ests, walls, threads = [], [], 1
    for _ in range(args.steps):
        est, wall, threads = cpu_sample(img, mask, p, iters)
        ests.append(est)
        walls.append(wall)
    est = statistics.median(ests)
    value = mpix / est
    calib = cpu_calibration()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(walls), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (reference arithmetic)", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": workload_desc(), "path": "reference algorithm on host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "per step: 1 PatchMatch (OpenMP) + 1 NL-Poisson update on each of the 8 scales, "
                                   "scaled by the per-scale call counts of the %s; estimated %.1f s per "
                                   "process()" % (source, est),
                         "flags": TIMING_FLAGS, "calibration": calib},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    pkg = ge.package()
    ge.build() if not os.path.exists(pkg.LIB_PATH) else None
    ctx = pkg.Context(local)
    if args.pm_variant is not None:
        ctx.set_tuning(ctx.TUNE_PM_VARIANT, args.pm_variant)
    if args.cg_precond is not None:
        ctx.set_tuning(ctx.TUNE_CG_PRECOND, args.cg_precond)
    if args.pm_bound is not None:
        ctx.set_tuning(ctx.TUNE_PM_BOUND, args.pm_bound)
    if args.batch_groups is not None:
        ctx.set_tuning(ctx.TUNE_BATCH_GROUPS, args.batch_groups)
    if args.pm_tile is not None:
        ctx.set_tuning(ctx.TUNE_PM_TILE, args.pm_tile)
    if args.graph_loop is not None:
        ctx.set_tuning(ctx.TUNE_GRAPH_LOOP, args.graph_loop)
    img, mask, p = workload()
    H, W, C = img.shape
    mpix = W * H / 1e6
    dev = "cuda:%d" % local
    d_img = torch.from_numpy(img).to(dev)
    d_mask = torch.from_numpy(mask).to(dev)
    d_out = torch.empty_like(d_img)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(fn, k, profile=False):
        ms = []
        for i in range(k):
            flush.fill_(i & 0xFF)  # evict L2 between steps (outside the timed events)
            torch.cuda.synchronize()
            barrier()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return ms

    seed = 1234 + rank

    def step():
        # the same seed every step: every step does the same work
        ctx.set_seed(seed)
        ctx.process_device(d_img, d_mask, p, out=d_out)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    clocks = Clocks(local)
    clocks.start()
    ms = timed(step, args.steps)
    clk = clocks.stop()
    launches = ctx.launch_count() - l0
    total_ms = max_over_ranks(sum(ms), dev)
    value = job_throughput(world, args.steps, mpix, total_ms)

    # the same steps again with per-kernel CUDA events (the kernel table and
    # the rooflines); events bracket every launch, so these steps run the
    # host iteration loop and are not the timed value
    c0 = ctx.counters()
    ctx.set_profiling(True)
    pms = timed(step, args.steps)
    prof = ctx.profile()
    ctx.set_profiling(False)
    c1 = ctx.counters()
    prof_total_ms = sum(pms)

    # end to end: pinned host buffers, copies inside the timed region
    import ctypes as ct
    h_img = torch.from_numpy(img).pin_memory()
    h_mask = torch.from_numpy(mask).pin_memory()
    h_out = torch.empty_like(h_img).pin_memory()
    st = pkg.ProcessStats()

    def e2e_step():
        ctx.set_seed(seed)
        rc = ctx.lib.nli_process(ctx.h, ct.byref(p), ct.c_void_p(h_img.data_ptr()), ct.c_void_p(h_mask.data_ptr()),
                                 W, H, C, ct.c_void_p(h_out.data_ptr()), ct.byref(st))
        if rc != 0:
            raise RuntimeError(ctx.lib.nli_last_error(ctx.h).decode())

    e2e_step()
    ems = timed(e2e_step, args.steps)
    e_total = max_over_ranks(sum(ems), dev)
    e2e_value = job_throughput(world, args.steps, mpix, e_total)

    # the same steps with the Jacobi-preconditioned CG (NLI_TUNE_CG_PRECOND = 1):
    # the plain CG's stopping test on the true residual, fewer iterations, a
    # solution that differs from the reference's within the CG tolerance
    jacobi = None
    if world == 1 and args.cg_precond is None and not args.no_variants:
        ctx.set_tuning(ctx.TUNE_CG_PRECOND, 1)
        try:
            step()
            torch.cuda.synchronize()
            k0 = ctx.counters()["cg_iterations"]
            jms = timed(step, args.steps)
            k1 = ctx.counters()["cg_iterations"]
        finally:
            ctx.set_tuning(ctx.TUNE_CG_PRECOND, 0)
        jacobi = {"value": job_throughput(world, args.steps, mpix, sum(jms)), "unit": UNIT,
                  "ms_per_step": sum(jms) / args.steps, "cg_iterations_per_step": (k1 - k0) / args.steps,
                  "path": "plain process(), inputs resident, Jacobi-preconditioned CG"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    batch = None if (args.batch_count <= 0 or world > 1) else batch_compare(pkg, ctx, args, local)

    # roofline of the dominant kernel, from the events timed inside the steps
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s: FP32 lanes x FMA at the sampled clock
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (0, 0.0))
    cand = c1["candidates"] - c0["candidates"]
    pm_ms = sum(v[1] for k, v in prof.items() if k.startswith("pm_"))
    pm_launches = sum(v[0] for k, v in prof.items() if k.startswith("pm_"))
    traffic = None
    if WORKLOAD == "nlpoisson512" and os.path.exists(TRAFFIC):
        import re
        m = re.search(r"traffic_bytes_per_launch:\s*(\d+)", open(TRAFFIC).read())
        traffic = int(m.group(1)) if m else None
    stats = st.as_dict()
    formula = formula_candidates(stats, p.patchmatch.iterations) * args.steps
    pm_tflops = formula * flop_per_candidate() / (pm_ms / 1e3) / 1e12 if pm_ms > 0 else 0.0
    eval_tflops = cand * flop_per_candidate() / (pm_ms / 1e3) / 1e12 if pm_ms > 0 else 0.0
    roofline = {"kernel": "k_pm_init + k_pm_sweep (PatchMatch)", "bound": "fp32", "achieved": pm_tflops,
                "peak": fp32_peak, "unit": "TFLOP/s", "frac": pm_tflops / fp32_peak if fp32_peak else None,
                "traffic": traffic, "traffic_scope": "ncu DRAM bytes of one finest-scale (512x512) sweep launch",
                "launches": pm_launches, "ms": pm_ms,
                "peak_source": "nominal FP32 (%d SMs x 128 lanes x 2 FLOP) at the sampled median SM clock %.0f MHz; "
                               "MEASURED_PEAKS.json has no FP32 figure" % (n_sm, sm_mhz),
                "flop_per_candidate": flop_per_candidate(),
                "work": "algorithmic: the reference's candidates by the hot-path formula, per PatchMatch call "
                        "N_t (1 + I (2 + W_rs)), summed over the run's calls",
                "formula_candidates": formula,
                "evaluated_candidates": cand,
                "evaluated_tflops": eval_tflops,
                "evaluated_note": "candidates the kernels evaluated (the patch-mean lower bound skips the rest), "
                                  "each counted at the full 2519 FLOP though %.1f %% of them stopped after 4 of "
                                  "10 rows" % (100.0 * (c1["candidates_partial"] - c0["candidates_partial"])
                                                / max(cand, 1))}
    cg = prof.get("poisson_cg", (0, 0.0))
    cg_work = c1["cg_unknown_iterations"] - c0["cg_unknown_iterations"]
    cg_gbs = cg_work * CG_BYTES_PER_UNKNOWN_ITER / (cg[1] / 1e3) / 1e9 if cg[1] > 0 else 0.0
    kernels = {k: {"launches": v[0], "ms": v[1], "share": v[1] / prof_total_ms if prof_total_ms else None}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        iters, source = reference_counts()
        if iters is None:
            iters, source = list(st.iterations[:p.scales]), "GPU run (no reference counts for this workload)"
        est, wall, threads = cpu_sample(img, mask, p, iters)
        method = {0: "NL-means", 1: "NL-medians", 2: "NL-Poisson", 3: "NL-depth"}.get(p.update.method, "update")
        cpu = {"value": mpix / est, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "1 PatchMatch (OpenMP) + 1 %s update on each of the %d scales (%.1f s wall), scaled "
                         "by the per-scale call counts of the %s: %.1f s per process()"
                         % (method, p.scales, wall, source, est),
               "flags": TIMING_FLAGS, "calibration": cpu_calibration()}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 CG inner products)", "data": "synthetic",
        "config": {"workload": workload_desc(), "path": "plain (one process() per step)",
                   "iteration_loop": "iterations after a scale's first in one CUDA graph per scale (while node, "
                                     "stopping test on the device)" if ctx.get_tuning(ctx.TUNE_GRAPH_LOOP)
                                     else "host loop",
                   "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas x%d" % world},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(img.nbytes + mask.nbytes),
                "d2h_bytes_per_step": int(img.nbytes), "ms_per_step": e_total / args.steps},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roofline,
        "roofline_cg": {"kernel": "k_poisson_cg", "bound": "hbm", "achieved": cg_gbs, "peak": hbm_peak,
                        "unit": "GB/s", "frac": cg_gbs / hbm_peak if hbm_peak else None,
                        "bytes_per_unknown_iteration": CG_BYTES_PER_UNKNOWN_ITER, "peak_source": "measured"},
        "kernels": kernels,
        "kernels_pass": {"ms_per_step": prof_total_ms / args.steps,
                         "note": "the kernel table and rooflines come from a second pass of the same steps with "
                                 "per-kernel CUDA events (host iteration loop)"},
        "dominant_kernel": dom[0],
        "cpu_baseline": cpu,
        "batched": batch,
        "process_stats": {"iterations": list(st.iterations[:p.scales]), "patchmatch_calls": st.patchmatch_calls,
                          "update_calls": st.update_calls, "cg_iterations": st.cg_iterations},
        "cg_jacobi": jacobi,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def hole_psnr(out, truth, mask):
    """PSNR (peak 255) over the hole pixels and channels."""
    m = np.asarray(mask) > 0
    d = np.asarray(out, np.float64)[m] - np.asarray(truth, np.float64)[m]
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0 else 10.0 * np.log10(255.0 ** 2 / mse)


def batch_reference_gaps(items5, outs, batch=(5, 64, 1024)):
    """Hole PSNR against the truth (the input's hole pixels) of our outputs
    and of the reference's (tests/golden/batch_reference_*.npz, made by
    tests/golden/make_golden.py --batch) for the batch items that have
    one; gap = ours - reference (dB).  batch = (seed, count, largest side)
    of the batch `items5` is: only references of that batch compare."""
    import glob
    rows = []
    for path in sorted(glob.glob(os.path.join(GOLDEN, "batch_reference_*.npz"))):
        g = np.load(path)
        i = int(g["index"])
        if i >= len(outs) or tuple(int(v) for v in g["batch"]) != tuple(batch):
            continue
        img, mask = items5[i][0], items5[i][1]
        truth = img[mask > 0].astype(np.float64)
        ref = g["hole"].astype(np.float64)
        p_ref = 10.0 * np.log10(255.0 ** 2 / float(np.mean((ref - truth) ** 2)))
        p_ours = hole_psnr(outs[i], img, mask)
        rows.append({"index": i, "size": [int(img.shape[1]), int(img.shape[0])], "method": items5[i][2],
                     "psnr_ours_db": p_ours, "psnr_reference_db": p_ref, "gap_db": p_ours - p_ref})
    return rows


def batch_compare(pkg, ctx, args, local):
    """Plain per-image path against the batched path on the uneven-batch
    workload: `--batch-count` images (64), sides log-uniform in [128,
    --batch-max-side (1024)], aspect 0.5-2, 5-30 % ellipse or stroke holes,
    alternating nlmeans / nlpoisson, patch 9, scales
    |round(log(size 0.1) / log(0.75))| with the automatic coarsest rate.
    Inputs resident in HBM; the batched path (lockstep) runs once untimed
    (it sizes its workspace) and once timed, the plain path once timed, each
    with CUDA events on the context's stream.  Outputs are compared bit for
    bit, and the hole PSNR of the items with a reference output is compared
    with the reference's."""
    import torch
    from nli_gb300 import workloads as wl
    items5 = wl.config5(seed=5, count=args.batch_count, max_side=args.batch_max_side)
    items, params, mpix = [], [], 0.0
    for img, mask, method, scales in items5:
        items.append((ctx._f32(img), ctx._u8(mask)))
        params.append(wl.config5_params(mask, method, scales))
        mpix += img.shape[0] * img.shape[1] / 1e6
    outs = [torch.empty_like(i) for i, _ in items]
    ref = [torch.empty_like(i) for i, _ in items]
    seed = 2024

    def plain():
        for i, ((im, m), p) in enumerate(zip(items, params)):
            ctx.set_seed(ctx.batch_seed(seed, i))
            ctx.process_device(im, m, p, out=ref[i])

    def batched(mode=1):
        ctx.set_seed(seed)
        ctx.set_tuning(ctx.TUNE_BATCH_MODE, mode)
        ctx.set_batch_width(args.batch_width)
        try:
            ctx.process_batch_device(items, params, outs=outs)
        finally:
            ctx.set_tuning(ctx.TUNE_BATCH_MODE, 1)

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    batched()
    l0 = ctx.launch_count()
    tb = timed(batched)
    launches = ctx.launch_count() - l0
    tp = timed(plain)
    identical = all(bool(torch.equal(x, y)) for x, y in zip(outs, ref))
    by_groups = None
    if args.batch_groups_sweep:
        # the lockstep batch per number of concurrent sub-groups
        by_groups = {}
        keep = ctx.get_tuning(ctx.TUNE_BATCH_GROUPS)
        try:
            for g in (1, 2, 4):
                ctx.set_tuning(ctx.TUNE_BATCH_GROUPS, g)
                batched()
                by_groups[str(g)] = round(timed(batched), 3)
                identical = identical and all(bool(torch.equal(x, y)) for x, y in zip(outs, ref))
        finally:
            ctx.set_tuning(ctx.TUNE_BATCH_GROUPS, keep)
    workers = None
    if args.batch_workers:
        batched(0)
        tw = timed(lambda: batched(0))
        workers = {"mpix_s": mpix / tw, "s": tw, "batch_width": args.batch_width,
                   "identical_to_plain": all(bool(torch.equal(x, y)) for x, y in zip(outs, ref)),
                   "path": "worker contexts (NLI_TUNE_BATCH_MODE 0): whole process() runs on their own streams"}

    def kernel_ms(fn):
        # one more pass with per-kernel CUDA events (outside the timed passes)
        ctx.set_profiling(True)
        fn()
        prof = ctx.profile()
        ctx.set_profiling(False)
        return {k: round(v[1], 1) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    kb, kp = (kernel_ms(batched), kernel_ms(plain)) if args.batch_profile else (None, None)
    host = [o.cpu().numpy() for o in ref]
    gaps = batch_reference_gaps(items5, host, (5, args.batch_count, args.batch_max_side))
    return {"workload": "uneven batch: %d images, sides log-uniform 128-%d, aspect 0.5-2, 5-30%% ellipse/stroke "
                        "holes, nlmeans/nlpoisson alternating, patch 9, scales |round(log(0.1 size)/log(0.75))|, "
                        "automatic coarsest rate (seed 5)" % (len(items), args.batch_max_side),
            "mpix": mpix, "plain_mpix_s": mpix / tp, "batched_mpix_s": mpix / tb, "speedup": tp / tb,
            "plain_s": tp, "batched_s": tb, "batch_groups": ctx.get_tuning(ctx.TUNE_BATCH_GROUPS),
            "batched_s_by_groups": by_groups,
            "batched_path": "lockstep: one launch per kernel per pyramid rank over every image, each rank's "
                            "iteration loop one CUDA graph (while node, per-image stopping test on the device); "
                            "the images dealt into concurrent sub-groups on worker contexts",
            "plain_path": "one process() per image, iterations after a scale's first in one CUDA graph",
            "gpu_launches": int(launches), "identical_to_plain": identical,
            "reference_psnr": gaps,
            "max_psnr_gap_db": max((-r["gap_db"] for r in gaps), default=None),
            "mean_psnr_gap_db": float(np.mean([r["gap_db"] for r in gaps])) if gaps else None,
            "workers": workers, "kernel_ms_plain": kp, "kernel_ms_batched": kb,
            "scales": [p.scales for p in params]}


def run_case(args):
    """Cases for profiler captures: one PatchMatch call (init + 10 sweeps) or
    one NL-Poisson update on the finest scale of the benchmark workload, with
    the masks the driver builds there; or whole process() calls (`process`,
    the launch sequence of one benchmark step per --steps)."""
    import torch
    pkg = ge.package()
    ctx = pkg.Context(0)
    if args.pm_variant is not None:
        ctx.set_tuning(ctx.TUNE_PM_VARIANT, args.pm_variant)
    if args.cg_precond is not None:
        ctx.set_tuning(ctx.TUNE_CG_PRECOND, args.cg_precond)
    if args.pm_bound is not None:
        ctx.set_tuning(ctx.TUNE_PM_BOUND, args.pm_bound)
    if args.batch_groups is not None:
        ctx.set_tuning(ctx.TUNE_BATCH_GROUPS, args.batch_groups)
    if args.pm_tile is not None:
        ctx.set_tuning(ctx.TUNE_PM_TILE, args.pm_tile)
    if args.graph_loop is not None:
        ctx.set_tuning(ctx.TUNE_GRAPH_LOOP, args.graph_loop)
    ctx.set_seed(7)
    img, mask, p = workload()
    if args.case == "batch":
        # one lockstep batch of the uneven-batch workload (--batch-count
        # images, sides up to --batch-max-side), --steps times
        from nli_gb300 import workloads as wl
        items5 = wl.config5(seed=5, count=args.batch_count, max_side=args.batch_max_side)
        items = [(ctx._f32(i), ctx._u8(m)) for i, m, _, _ in items5]
        params = [wl.config5_params(m, meth, sc) for _, m, meth, sc in items5]
        l0 = ctx.launch_count()
        for _ in range(args.steps):
            ctx.set_seed(2024)
            ctx.process_batch_device(items, params)
        torch.cuda.synchronize()
        print(json.dumps({"case": "batch", "images": len(items), "launches": ctx.launch_count() - l0,
                          "counters": ctx.counters()}))
        return 0
    if args.case == "process":
        d_img, d_mask = ctx._f32(img), ctx._u8(mask)
        d_out = torch.empty_like(d_img)
        l0 = ctx.launch_count()
        for _ in range(args.steps):
            ctx.set_seed(1234)
            _, st = ctx.process_device(d_img, d_mask, p, out=d_out)
        torch.cuda.synchronize()
        print(json.dumps({"case": "process", "launches": ctx.launch_count() - l0, "stats": st}))
        return 0
    ext = ctx.extended_domain(mask, p.update.patch_x, p.update.patch_y)
    src, tgt, _ = ctx.scale_masks(ext, p.update.patch_x // 2, True)
    d_img = ctx._f32(img)
    d_img[torch.from_numpy(mask).to(d_img.device).bool()] = 128.0
    nnf = None
    for _ in range(args.steps):
        nnf, _, e = ctx.patchmatch(p.distance, p.patchmatch, d_img, src, d_img, tgt, init=nnf)
    if args.case == "update":
        conf = ctx.confidence_mask(mask, p.conf_decay_time, p.conf_asymptotic)
        for _ in range(args.steps):
            out, tot = ctx.update(p.update, d_img, d_img, mask, ext, nnf, conf)
    torch.cuda.synchronize()
    print(json.dumps({"case": args.case, "energy": e, "counters": ctx.counters()}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default=None, choices=["patchmatch", "update", "process", "batch"],
                    help="run one small profiling case instead of the benchmark")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--pm-variant", type=int, default=None, choices=[0, 1, 2],
                    help="9x9 PatchMatch window reads: 0 target in shared memory + plain source loads, "
                         "1 source windows staged by tensor copies, 2 target in registers "
                         "(default: the library's)")
    ap.add_argument("--workload", default="nlpoisson512", choices=sorted(WORKLOADS),
                    help="nlpoisson512 (the headline, default), nlmeans256 or nldepth640")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the extra measurement with the Jacobi-preconditioned CG")
    ap.add_argument("--cg-precond", type=int, default=None, choices=[0, 1],
                    help="NL-Poisson CG: 0 plain (the reference's), 1 Jacobi-preconditioned "
                         "(default: the library's, 0)")
    ap.add_argument("--pm-bound", type=int, default=None, choices=[0, 1, 2],
                    help="PatchMatch lower bound: 1 patch means, 2 means and deviations, 0 every candidate "
                         "evaluated (default: the library's, 1)")
    ap.add_argument("--pm-tile", type=int, default=None,
                    help="PatchMatch work distribution: 0 static block ranges, n > 0 a device work queue of n "
                         "target points per grab (default: the library's, 1)")
    ap.add_argument("--graph-loop", type=int, default=None, choices=[0, 1, 2],
                    help="iteration loops as CUDA graphs: 1 plain runs and lockstep batches, 2 also worker "
                         "batches, 0 host loops (for profilers that cannot see into conditional graphs); "
                         "default: the library's, 1")
    ap.add_argument("--batch-groups", type=int, default=None,
                    help="concurrent sub-groups of a lockstep batch group (default: the library's, 2)")
    ap.add_argument("--batch-count", type=int, default=64,
                    help="images in the batched-vs-plain comparison (0 skips it)")
    ap.add_argument("--batch-max-side", type=int, default=1024)
    ap.add_argument("--batch-width", type=int, default=8,
                    help="images in flight in the worker-context batch form")
    ap.add_argument("--batch-profile", action="store_true",
                    help="add per-kernel profiled passes of both paths to the batch comparison")
    ap.add_argument("--no-batch-profile", dest="batch_profile", action="store_false")
    ap.add_argument("--batch-groups-sweep", action="store_true",
                    help="also time the lockstep batch with 1, 2 and 4 concurrent sub-groups")
    ap.add_argument("--batch-workers", action="store_true",
                    help="also time the worker-context batch form (NLI_TUNE_BATCH_MODE 0)")
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = args.workload
    if args.case:
        return run_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
