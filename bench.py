#!/usr/bin/env python3
"""Benchmark driver.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload pt|kd|serve|relmse|bpt]

Prints ONE JSON line (rank 0).  Workloads:

  pt  (default) path tracing of the mixed-material scene as configured: 25
      displaced level-5 icospheres (512,006 triangles) on a ground plane,
      40 % diffuse / 40 % isotropic Phong / 20 % refractive, two area lights,
      1024x1024 at 256 samples per pixel, max path length 16.  One step = one
      wr_render_device call of the whole configuration (268,435,456 paths)
      through the wavefront renderer with the reference's estimator, in the
      configuration wr_autotune picks first.  Metric: Mpaths/s.  Beside it:
      the plain megakernel on the same call, the time to relMSE 1e-3 of both
      renderers with the reference's estimator and with the low-variance one
      (NEE with MIS + mirror-lobe Phong), the extend stage's roofline, and --
      unless --no-extras -- the kd microbenchmark (key "kd") and a short
      serving stream (key "serve").
  kd  closest-hit microbenchmark: level-8 displaced icosphere (1,310,720
      triangles), 2^24 rays; one step = all rays.  Metric: Mrays/s.
  serve  a seeded Poisson stream of render requests through the serving
      loop (20 requests/s for 60 s; 10 s inside the default line): p50 / p99
      latency, slowdowns and Mpaths/s, at that rate and slowed to 60 % load.
  relmse relMSE of each path-tracing configuration at its own spp against a
      converged image (configuration 0: the reference's 16,384-spp CPU image).
  bpt bidirectional path tracing (WR_MODE_BIDIRECTIONAL) of the Cornell box,
      256x256, max path length 8; one step = one render call of 16 samples
      per pixel (1,048,576 eye + light sub-path pairs, all connections).
      Metric: Msamples/s (the unidirectional megakernel, vertex connection
      and merging, WR_MODE_VCM, and progressive photon mapping,
      WR_MODE_PHOTON_MAP, both with base radius 0.01, on the same scene
      beside it).

`value` is device-timed with CUDA events per step on the launching stream,
with the L2 flushed (a 512 MiB write) before every step and inputs resident
in HBM; `e2e` runs the same steps through the public C ABI with host buffers
(wr_render returning the image to the host / wr_trace_closest with pinned
host rays and hits), host<->device copies inside the timed region.
`--impl reference` times WalkRay's CPU algorithm (the C restatement of it,
all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# Per-ray traversal work of the reference on the kd workload (2^24 rays,
# seed 1), counted by the oracle (`wr_oracle count`, asserted in
# tests/test_trace_gpu.py): AABB tests and ray-triangle tests per ray.
KD_BOX_TESTS = 22.5567
KD_TRI_TESTS = 2.9383
# algorithmic bytes of one traced ray: ray in (24) + hit out (16) + per box
# test 8 B topology + 24 B AABB + per triangle test 3 x 16 B vertices + 4 B id
RAY_IO_BYTES, BOX_BYTES, TRI_BYTES = 40, 32, 52
KD_BYTES_PER_RAY = RAY_IO_BYTES + KD_BOX_TESTS * BOX_BYTES + KD_TRI_TESTS * TRI_BYTES
KD_WORKLOAD = "kd: level-8 displaced icosphere (1,310,720 tris), 2^24 rays (origins in 2x bounds, uniform directions)"

PT_SIZE, PT_DEPTH, PT_SEED = 1024, 16, 7
PT_SPP = 256  # samples per pixel per step: one render call of the whole configuration
METRIC_PT = "Mpaths/s (wavefront path tracing, 1024^2 mixed-material scene; time-to-relMSE 1e-3 beside it)"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines: list[str] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce(world, x: float, op: str) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def timed_steps(step, k: int, stream, flush):
    """Sum of per-step CUDA-event durations (ms) on `stream`, L2 flushed before each step."""
    import torch

    evs = []
    with torch.cuda.stream(stream):
        for i in range(k):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step(i)
            b.record(stream)
            evs.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs)


def launches(ctx) -> int:
    import ctypes as C

    v = C.c_uint64()
    ctx.lib.wr_kernel_launches(ctx.h, C.byref(v))
    return v.value


# ---------------------------------------------------------------------------
# pt: wavefront path tracing of the mixed-material scene
# ---------------------------------------------------------------------------
def pt_scene():
    from walkray_gb300 import scenes as S

    return S.mixed_spheres(PT_SIZE, PT_SIZE, seed=PT_SEED)


def relmse_per_sample(s1, s2, spp, ref):
    """relMSE of a 1-spp image against the converged image R: mean over pixels
    and channels of Var/(R^2 + 1e-2), with the per-sample variance of each
    pixel from its sum s1 and sum of squares s2 over `spp` samples (the
    estimator is unbiased, so MSE = variance and an n-spp image has 1/n of
    it).  Also the share of the total that comes from the top 0.1 % of
    entries: a large share means a heavy-tailed estimator."""
    var = np.maximum(s2 / spp - (s1 / spp) ** 2, 0.0) * spp / (spp - 1)
    e = var / (ref ** 2 + 1e-2)
    top = np.sort(e.ravel())[::-1][: max(1, e.size // 1000)]
    return float(e.mean()), float(top.sum() / max(e.sum(), 1e-30))


def cpu_baseline_pt(scene, rows: int, threads: int):
    import wr_oracle

    w = scene.camera.width
    y0 = (scene.camera.height - rows) // 2
    orc = wr_oracle.SceneOracle(scene)
    t0 = time.perf_counter()
    orc.render(1, PT_DEPTH, seed=1, p0=y0 * w, p1=(y0 + rows) * w, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": rows * w / dt / 1e6, "unit": "Mpaths/s", "cores": threads, "kind": "port",
            "sample": f"{rows} centre rows x {w} pixels x 1 spp of the 1024^2 mixed-material scene, "
                      f"WalkRay's PathTracer restated in C (oracle), {threads} OpenMP threads, tree build excluded"}


def time_to_relmse(ctx, sid, flags, ms_per_spp):
    """Time to relMSE 1e-3 of one estimator: per-pixel variance from 64 spp
    (sum and sum of squares) against R, an independent 256-spp image of the
    low-variance estimator (the least noisy reference at hand; an unbiased
    estimator's MSE is its variance, so relMSE(n spp) = rel_1spp / n)."""
    from walkray_gb300.api import LOW_VARIANCE

    ref = ctx.render(sid, 256, PT_DEPTH, seed=99, mode="wavefront", flags=LOW_VARIANCE).astype(np.float64)
    s1, s2 = ctx.render_stats(sid, 64, PT_DEPTH, seed=11, mode="wavefront", flags=flags)
    rel1, top_share = relmse_per_sample(s1, s2, 64, ref)
    spp_needed = rel1 / 1e-3
    out = {"spp_needed": round(spp_needed, 1), "relmse_1spp": round(rel1, 5),
           "share_of_top_0.1pct_entries": round(top_share, 4)}
    for k, v in ms_per_spp.items():
        out[k + "_s"] = round(spp_needed * v / 1e3, 3)
    return out


def run_pt(args, world, rank, local):
    import torch

    from walkray_gb300.api import LOW_VARIANCE, Context

    torch.cuda.set_device(local)
    scene = pt_scene()
    npix = PT_SIZE * PT_SIZE
    ctx = Context(device=local)
    sid = ctx.upload(scene)
    tuned = ctx.autotune(sid, 16, PT_DEPTH) if not args.no_tune else None
    stream = torch.cuda.Stream()
    film = torch.zeros(npix * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    seed = 1000 + rank
    mk_steps = max(1, min(args.steps, args.mk_steps))

    def step_mode(mode, flags=0):
        return lambda i: ctx.render_device(sid, PT_SPP, PT_DEPTH, film.data_ptr(), seed=seed, mode=mode,
                                           spp_offset=i * PT_SPP, stream=stream.cuda_stream, flags=flags)

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step_mode("wavefront")(i)
        step_mode("megakernel")(0)
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clk:
        l0 = launches(ctx)
        ms = timed_steps(step_mode("wavefront"), args.steps, stream, flush)
        n_launch = launches(ctx) - l0
        ms_mk = timed_steps(step_mode("megakernel"), mk_steps, stream, flush)
    ms_max = allreduce(world, ms, "max")
    paths = float(npix * PT_SPP * args.steps)
    units = allreduce(world, paths, "sum")
    value = units / (ms_max / 1e3) / 1e6
    mk_value = allreduce(world, float(npix * PT_SPP * mk_steps), "sum") / (allreduce(world, ms_mk, "max") / 1e3) / 1e6

    # e2e: wr_render returning the image to the host, PT_SPP samples per pixel per step
    barrier(world)
    t0 = time.perf_counter()
    for i in range(args.steps):
        ctx.render(sid, PT_SPP, PT_DEPTH, seed=seed + 1, mode="wavefront", spp_offset=i * PT_SPP)
    e2e_s = allreduce(world, time.perf_counter() - t0, "max")
    e2e = allreduce(world, paths, "sum") / e2e_s / 1e6

    line = {
        "metric": METRIC_PT, "value": round(value, 2), "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": pt_workload(),
                   "renderer": "wavefront (generate/extend/shade/shadow queues, CUDA-graph bounce loop)",
                   "l2": "flushed (512 MiB write) before every step", "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e, 2), "unit": "Mpaths/s", "h2d_bytes_per_step": 256 + 4 * 257,
                "d2h_bytes_per_step": npix * 12},
        "megakernel": {"value": round(mk_value, 2), "unit": "Mpaths/s", "ms_per_step": round(ms_mk / mk_steps, 3),
                       "steps": mk_steps},
        "paths_per_step": npix * PT_SPP,
        "wavefront_over_megakernel": round(value / mk_value, 3),
        "gpu_launches": int(n_launch), "clocks": clk.summary(),
    }
    if tuned:
        line["config"]["autotuned"] = {k: tuned[k] for k in ("capacity", "extend_block", "shade_block",
                                                             "ctas_per_sm", "iters_per_graph", "refill_min",
                                                             "leaf_min", "steps_per_turn", "pixel_tile")}
        line["config"]["autotuned"]["trial_mpaths_per_s"] = round(tuned["mpaths_per_s"], 1)
        line["config"]["autotuned"]["how"] = ("wr_autotune: coordinate descent from the defaults, 16-spp trial "
                                              "renders of this scene")
    if rank == 0 and not args.quick:
        # roofline of the dominant kernel (the extend / traversal stage), from a
        # profiled render of one step.  Algorithmic bytes count the reference's
        # traversal work (every box and triangle KDTree::intersect visits: the
        # same render with WR_RENDER_EXACT_TRAVERSAL); the time is that of the
        # default (pruned) extend stage.
        prof = ctx.profile_render(sid, PT_SPP, PT_DEPTH, film.data_ptr(), seed=seed + 2)
        refw = ctx.profile_render(sid, PT_SPP, PT_DEPTH, film.data_ptr(), seed=seed + 2, exact=True)
        peak, peak_kind = peaks()
        alg = refw["rays"] * RAY_IO_BYTES + refw["box_tests"] * BOX_BYTES + refw["tri_tests"] * TRI_BYTES
        achieved = alg / (prof["ms_extend"] / 1e3) / 1e9
        traffic = None
        pf = os.path.join(ROOT, "profiles", "wf_extend_pt.json")
        if os.path.exists(pf):
            per_ray = json.load(open(pf)).get("dram_bytes_per_ray")
            traffic = round(per_ray * prof["rays"] / max(1, prof["iterations"]), 0) if per_ray else None
        nr = max(1, refw["rays"])
        line["roofline"] = {
            "bound": "hbm", "kernel": "k_wf_extend", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
            "algorithmic_bytes_per_ray": round(alg / nr, 1),
            "reference_box_tests_per_ray": round(refw["box_tests"] / nr, 3),
            "reference_tri_tests_per_ray": round(refw["tri_tests"] / nr, 3),
            "executed_box_tests_per_ray": round(prof["box_tests"] / max(1, prof["rays"]), 3),
            "executed_tri_tests_per_ray": round(prof["tri_tests"] / max(1, prof["rays"]), 3),
            "stage_ms": {k: round(prof[k], 2) for k in ("ms_extend", "ms_shade", "ms_shadow", "ms_generate")},
            "rays_per_step": prof["rays"], "iterations": prof["iterations"],
            "rays_per_s_extend": round(prof["rays"] / (prof["ms_extend"] / 1e3) / 1e6, 1),
        }
        # time to relMSE 1e-3 with the reference's estimator and with the
        # low-variance one; each estimator's own throughput on both renderers
        lv_steps = max(1, min(3, args.steps))
        with torch.cuda.stream(stream):
            step_mode("wavefront", LOW_VARIANCE)(0)
            step_mode("megakernel", LOW_VARIANCE)(0)
        ms_lv = timed_steps(step_mode("wavefront", LOW_VARIANCE), lv_steps, stream, flush)
        ms_lv_mk = timed_steps(step_mode("megakernel", LOW_VARIANCE), lv_steps, stream, flush)
        per = {"reference_estimator": {"wavefront": ms / args.steps / PT_SPP,
                                       "megakernel": ms_mk / mk_steps / PT_SPP},
               "low_variance_estimator": {"wavefront": ms_lv / lv_steps / PT_SPP,
                                          "megakernel": ms_lv_mk / lv_steps / PT_SPP}}
        ttr = {}
        for name, f in (("reference_estimator", 0), ("low_variance_estimator", LOW_VARIANCE)):
            ttr[name] = time_to_relmse(ctx, sid, f, per[name])
            ttr[name]["mpaths_per_s"] = {k: round(npix / v / 1e3, 2) for k, v in per[name].items()}
        ttr["formula"] = ("relMSE = mean((I-R)^2/(R^2+1e-2)) = mean(Var/(R^2+1e-2))/spp for an unbiased estimator; "
                          "Var per pixel from 64 spp (sum, sum of squares), R = independent 256-spp wavefront image "
                          "with the low-variance estimator; time = spp needed x measured ms per spp")
        ttr["low_variance"] = "WR_RENDER_NEE_MIS | WR_RENDER_PHONG_MIRROR (same expectation as the reference's)"
        ttr["plain_megakernel_reference_estimator_over_wavefront_low_variance"] = round(
            ttr["reference_estimator"]["megakernel_s"] / ttr["low_variance_estimator"]["wavefront_s"], 1)
        line["time_to_relmse_1e-3"] = ttr
        if world == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline_pt(scene, args.cpu_rows or 64, os.cpu_count() or 1)
    ctx.close()
    return line


def pt_workload():
    return ("pt: 25 displaced level-5 icospheres (512,006 tris) on a ground plane, 40% diffuse / 40% Phong / "
            f"20% refractive, two area lights, {PT_SIZE}x{PT_SIZE}, max depth 16, {PT_SPP} spp per step (one render "
            "call), the reference's estimator")


def reference_pt(args):
    scene = pt_scene()
    threads = os.cpu_count() or 1
    rows = args.cpu_rows or 16
    for _ in range(min(args.warmup, 1)):
        cpu_baseline_pt(scene, 2, threads)
    vals = [cpu_baseline_pt(scene, rows, threads) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    return {"metric": METRIC_PT, "value": round(v, 4), "unit": "Mpaths/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": pt_workload(), "parallelism": "host cores of rank 0",
                       "sample_per_step": f"{rows} centre rows x {PT_SIZE} pixels x 1 spp ({rows * PT_SIZE} paths)"},
            "cpu_baseline": dict(vals[0], value=round(v, 4)),
            "e2e": {"value": round(v, 4), "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# bpt: the bidirectional renderer on the Cornell box
# ---------------------------------------------------------------------------
BPT_SIZE, BPT_DEPTH, BPT_SPP = 256, 8, 16
METRIC_BPT = "Msamples/s (bidirectional path tracing: eye + light sub-path pairs, all connections; Cornell 256^2)"


def bpt_scene():
    from walkray_gb300 import scenes as S

    return S.cornell(BPT_SIZE, BPT_SIZE)


def cpu_baseline_bpt(scene, spp: int, threads: int):
    import wr_oracle

    orc = wr_oracle.SceneOracle(scene)
    t0 = time.perf_counter()
    orc.render_bpt(spp, BPT_DEPTH, seed=1, threads=threads)
    dt = time.perf_counter() - t0
    n = BPT_SIZE * BPT_SIZE * spp
    return {"value": n / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{spp} spp of the {BPT_SIZE}^2 Cornell box ({n} samples), WalkRay's "
                      f"BidirectionalPathTracer restated in C (oracle), {threads} OpenMP threads, tree build excluded"}


def run_bpt(args, world, rank, local):
    import torch

    from walkray_gb300.api import Context

    torch.cuda.set_device(local)
    scene = bpt_scene()
    npix = BPT_SIZE * BPT_SIZE
    ctx = Context(device=local)
    sid = ctx.upload(scene)
    stream = torch.cuda.Stream()
    film = torch.zeros(npix * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    seed = 2000 + rank

    def step_mode(mode):
        return lambda i: ctx.render_device(sid, BPT_SPP, BPT_DEPTH, film.data_ptr(), seed=seed, mode=mode,
                                           spp_offset=i * BPT_SPP, stream=stream.cuda_stream)

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step_mode("bidirectional")(i)
            step_mode("megakernel")(i)
            step_mode("vcm")(i)
            step_mode("photon_map")(i)
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clk:
        l0 = launches(ctx)
        ms = timed_steps(step_mode("bidirectional"), args.steps, stream, flush)
        n_launch = launches(ctx) - l0
        ms_pt = timed_steps(step_mode("megakernel"), args.steps, stream, flush)
        ms_vcm = timed_steps(step_mode("vcm"), args.steps, stream, flush)
        ms_ppm = timed_steps(step_mode("photon_map"), args.steps, stream, flush)
    ms_max = allreduce(world, ms, "max")
    samples = float(npix * BPT_SPP * args.steps)
    value = allreduce(world, samples, "sum") / (ms_max / 1e3) / 1e6
    pt_value = allreduce(world, samples, "sum") / (allreduce(world, ms_pt, "max") / 1e3) / 1e6
    barrier(world)
    t0 = time.perf_counter()
    for i in range(args.steps):
        ctx.render(sid, BPT_SPP, BPT_DEPTH, seed=seed + 1, mode="bidirectional", spp_offset=i * BPT_SPP)
    e2e_s = allreduce(world, time.perf_counter() - t0, "max")
    e2e = allreduce(world, samples, "sum") / e2e_s / 1e6
    line = {
        "metric": METRIC_BPT, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (MIS products f64, as the reference)",
        "data": "synthetic (seeded scene generator)",
        "config": {"workload": bpt_workload(),
                   "l2": "flushed (512 MiB write) before every step", "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e, 3), "unit": "Msamples/s", "h2d_bytes_per_step": 256 + 4 * 257,
                "d2h_bytes_per_step": npix * 12},
        "unidirectional_megakernel": {"value": round(pt_value, 2), "unit": "Mpaths/s",
                                      "ms_per_step": round(ms_pt / args.steps, 3)},
        "vcm": {"value": round(allreduce(world, samples, "sum") / (allreduce(world, ms_vcm, "max") / 1e3) / 1e6, 3),
                "unit": "Msamples/s", "ms_per_step": round(ms_vcm / args.steps, 3), "base_radius": 0.01},
        "photon_map": {"value": round(allreduce(world, samples, "sum") / (allreduce(world, ms_ppm, "max") / 1e3) / 1e6,
                                      3),
                       "unit": "Msamples/s", "ms_per_step": round(ms_ppm / args.steps, 3), "base_radius": 0.01},
        "samples_per_step": npix * BPT_SPP, "gpu_launches": int(n_launch), "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_bpt(scene, args.cpu_rows or 2, os.cpu_count() or 1)
        import wr_oracle

        orc = wr_oracle.SceneOracle(scene)
        t0 = time.perf_counter()
        orc.render_vcm(1, BPT_DEPTH, seed=1, radius=0.01, threads=os.cpu_count() or 1)
        line["vcm"]["cpu_baseline"] = {"value": round(npix / (time.perf_counter() - t0) / 1e6, 4), "unit": "Msamples/s",
                                       "cores": os.cpu_count() or 1, "kind": "port",
                                       "sample": "1 spp, VCMTracer restated in C (oracle)"}
        t0 = time.perf_counter()
        orc.render_ppm(1, BPT_DEPTH, seed=1, radius=0.01, threads=os.cpu_count() or 1)
        line["photon_map"]["cpu_baseline"] = {"value": round(npix / (time.perf_counter() - t0) / 1e6, 4),
                                              "unit": "Msamples/s", "cores": os.cpu_count() or 1, "kind": "port",
                                              "sample": "1 spp, PhotonMap restated in C (oracle)"}
    ctx.close()
    return line


def bpt_workload():
    return (f"bpt: Cornell box {BPT_SIZE}x{BPT_SIZE}, max depth {BPT_DEPTH}, {BPT_SPP} spp per step (one render call), "
            "BidirectionalPathTracer semantics")


def reference_bpt(args):
    scene = bpt_scene()
    threads = os.cpu_count() or 1
    spp = args.cpu_rows or 1
    vals = [cpu_baseline_bpt(scene, spp, threads) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    return {"metric": METRIC_BPT, "value": round(v, 4), "unit": "Msamples/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": bpt_workload(), "parallelism": "host cores of rank 0",
                       "sample_per_step": f"{spp} spp of the {BPT_SIZE}x{BPT_SIZE} image"},
            "cpu_baseline": dict(vals[0], value=round(v, 4)),
            "e2e": {"value": round(v, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# serve: a seeded Poisson stream of render requests through the serving loop
# ---------------------------------------------------------------------------
SERVE_RATE = 20.0                       # requests per second
SERVE_RES = (128, 256, 512, 1024)       # square resolutions, drawn uniformly
SERVE_SPP = (16, 64, 256)
METRIC_SERVE = "request latency p50/p99 (s) and Mpaths/s, Poisson request stream through the serving loop"


def serve_scenes():
    """(name, scene, max path length): Cornell box, the mixed-material scene, the media scene."""
    from walkray_gb300 import scenes as S

    return [("cornell", S.cornell(256, 256), 8), ("mixed", S.mixed_spheres(1024, 1024, seed=PT_SEED), 16),
            ("media", S.cornell_media(512, 512), 24)]


def serve_stream(seconds: float, rate: float, seed: int):
    """Seeded arrivals: (time, scene index, side, spp), exponential gaps at `rate`."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            return out
        out.append((t, int(rng.integers(3)), SERVE_RES[rng.integers(4)], SERVE_SPP[rng.integers(3)]))


def run_stream(srv, sids, depths, stream):
    """Submits each request at its arrival time; returns per-request statuses (library clock)."""
    t0 = time.perf_counter()
    rids = []
    for (t, k, side, spp) in stream:
        dt = t - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        rids.append(srv.submit(sids[k], side, side, spp, depths[k], seed=len(rids) + 1))
    st = srv.wait(rids, timeout=3600)
    for r in rids:
        srv.fetch(r)
    return [st[r] for r in rids]


def serve_stats(stream, st, alone=None):
    """Latency = finish - submit on the library's clock.  `alone` (per
    request, seconds): its latency on an idle loop (the scene's latency
    floor plus its paths at the scene's throughput); slowdown = latency /
    alone (processor sharing at load rho gives about 1 / (1 - rho) to every
    request)."""
    lat = np.array([s["finish_s"] - s["submit_s"] for s in st])
    wait = np.array([s["admit_s"] - s["submit_s"] for s in st])
    paths = sum(s["paths_total"] for s in st)
    span = max(s["finish_s"] for s in st) - min(s["submit_s"] for s in st)
    out = {"requests": len(st), "p50_s": round(float(np.percentile(lat, 50)), 4),
           "p99_s": round(float(np.percentile(lat, 99)), 4),
           "p99_over_p50": round(float(np.percentile(lat, 99) / np.percentile(lat, 50)), 3),
           "mean_s": round(float(lat.mean()), 4),
           "admission_wait_p50_s": round(float(np.percentile(wait, 50)), 4),
           "mpaths_per_s": round(paths / span / 1e6, 2), "paths": int(paths), "makespan_s": round(span, 3),
           "offered_mpaths_per_s": round(paths / (stream[-1][0] if stream else 1.0) / 1e6, 2)}
    if alone is not None:
        sd = lat / np.maximum(np.asarray(alone), 1e-4)
        out["slowdown_p50"] = round(float(np.percentile(sd, 50)), 3)
        out["slowdown_p99"] = round(float(np.percentile(sd, 99)), 3)
        a = np.asarray(alone)
        out["alone_p99_over_p50"] = round(float(np.percentile(a, 99) / np.percentile(a, 50)), 2)
    return out


def run_serve(args, world, rank, local):
    import torch

    from walkray_gb300.api import Context, Server

    torch.cuda.set_device(local)
    scenes = serve_scenes()
    ctx = Context(device=local)
    sids = [ctx.upload(sc) for _, sc, _ in scenes]
    depths = [d for _, _, d in scenes]
    # per-sample relMSE of each (scene, resolution): variance of 16 spp per pixel
    # against an independent 64-spp image, mean of Var/(R^2 + 1e-2); a request
    # of s spp then has relMSE = that / s (unbiased estimator)
    rel1 = {}
    if not args.quick:
        for k, (name, sc, d) in enumerate(scenes):
            for side in SERVE_RES:
                sid = ctx.upload(scene_at(sc, side))
                s1, s2 = ctx.render_stats(sid, 16, d, seed=5, mode="wavefront")
                ref = ctx.render(sid, 64, d, seed=6, mode="wavefront").astype(np.float64)
                var = np.maximum(s2 / 16 - (s1 / 16) ** 2, 0) * 16 / 15
                rel1[(k, side)] = float(np.mean(var / (ref ** 2 + 1e-2)))
                ctx.release(sid)
    # each scene's throughput alone (a 512^2 x 64-spp render), for the slowdowns
    thr = []
    for k, (name, sc, d) in enumerate(scenes):
        sid = ctx.upload(scene_at(sc, 512))
        ctx.render(sid, 4, d, seed=1, mode="wavefront")
        t0 = time.perf_counter()
        ctx.render(sid, 64, d, seed=2, mode="wavefront")
        thr.append(512 * 512 * 64 / (time.perf_counter() - t0))
        ctx.release(sid)

    seconds = args.serve_seconds or (60.0 if args.workload == "serve" else 10.0)
    legs = {}
    stream = serve_stream(seconds, SERVE_RATE, seed=2024 + rank)
    pif = args.serve_capacity  # queue length while nobody waits for admission; 0 = the library's default (2^22)
    srv = Server(ctx, film_bytes=2 << 30, max_active=64, paths_in_flight=pif)
    run_stream(srv, sids, depths, [(0.0, k, 128, 16) for k in range(3)])  # warm-up: one small request per scene
    # the latency floor of each scene: its smallest request (128^2 x 16 spp) alone on the idle loop
    # (a path's bounces are graph replays, whatever the request's size)
    floor = []
    for k in range(3):
        lat = [(lambda s: s["finish_s"] - s["submit_s"])(run_stream(srv, sids, depths, [(0.0, k, 128, 16)])[0])
               for _ in range(3)]
        floor.append(float(np.median(lat)))

    def alone(stream):
        return [floor[k] + max(0, side * side * spp - 128 * 128 * 16) / thr[k] for (_, k, side, spp) in stream]

    with ClockSampler(local) as clk:
        st = run_stream(srv, sids, depths, stream)
    legs["stream"] = serve_stats(stream, st, alone(stream))
    legs["stream"]["slot_policy"] = "equal shares"
    if rel1:
        rr = [rel1[(k, side)] / spp for (_, k, side, spp) in stream]
        legs["stream"]["relmse_per_request"] = {"p50": float(np.percentile(rr, 50)), "max": float(max(rr))}
    # the same stream slowed to 60 % of the sustained throughput: latency without a backlog
    load = legs["stream"]["offered_mpaths_per_s"] / max(1e-9, legs["stream"]["mpaths_per_s"])
    f = load / 0.6
    slow = [(t * f, k, side, spp) for (t, k, side, spp) in stream]
    if load > 0.6 and not args.quick:
        st2 = run_stream(srv, sids, depths, slow)
        legs["stream_at_60pct_load"] = serve_stats(slow, st2, alone(slow))
        legs["stream_at_60pct_load"]["rate_req_per_s"] = round(SERVE_RATE / f, 3)
        legs["stream_at_60pct_load"]["slot_policy"] = "equal shares"
    srv.stop()
    if load > 0.6 and not args.quick and args.workload == "serve":
        fifo = Server(ctx, film_bytes=2 << 30, max_active=64, fifo=True, paths_in_flight=pif)
        run_stream(fifo, sids, depths, [(0.0, k, 128, 16) for k in range(3)])
        st3 = run_stream(fifo, sids, depths, slow)
        fifo.stop()
        legs["stream_at_60pct_load_fifo"] = serve_stats(slow, st3, alone(slow))
        legs["stream_at_60pct_load_fifo"]["rate_req_per_s"] = round(SERVE_RATE / f, 3)
        legs["stream_at_60pct_load_fifo"]["slot_policy"] = "admission order (WR_SERVE_FIFO)"
    ctx.close()
    main_leg = legs["stream"]
    line = {
        "metric": METRIC_SERVE, "value": main_leg["mpaths_per_s"], "unit": "Mpaths/s", "n_gpus": world,
        "steps": 1, "warmup": 1, "ms_per_step": round(main_leg["makespan_s"] * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes and arrivals)",
        "config": {"workload": f"serve: Poisson {SERVE_RATE:g} req/s for {seconds:g} s over Cornell (depth 8), "
                               "mixed-material (depth 16) and media (depth 24) scenes, resolution "
                               "U{128^2..1024^2}, spp U{16,64,256}", "parallelism": f"replicas x{world}"},
        "p50_s": main_leg["p50_s"], "p99_s": main_leg["p99_s"], "legs": legs, "clocks": clk.summary(),
        "queue_paths": {"no_request_waiting": args.serve_capacity or (1 << 22),
                        "requests_waiting": "the wavefront capacity (2^24 unless configured)"},
        "scene_mpaths_per_s_alone": [round(x / 1e6, 1) for x in thr],
        "scene_latency_floor_s": [round(x, 4) for x in floor],
        "slowdown": "latency / alone, alone = the scene's latency floor + the request's further paths at the "
                    "scene's throughput alone",
        "relmse_formula": "mean((I-R)^2/(R^2+1e-2)) = mean(Var/(R^2+1e-2))/spp, Var from 16 spp per pixel, "
                          "R = independent 64-spp image",
    }
    if rel1:
        line["relmse_1spp"] = {f"{scenes[k][0]}_{side}": round(v, 4) for (k, side), v in rel1.items()}
    return line


def scene_at(scene, side):
    """The same scene with a square camera of the given side."""
    import copy

    s = copy.copy(scene)
    c = s.camera
    # the image plane distance is in pixels: keep the field of view (as the serving loop does)
    ipd = float(np.float32(c.image_plane_dist) * np.float32(side / c.height))
    s.camera = dataclasses.replace(c, width=side, height=side, image_plane_dist=ipd)
    return s


# ---------------------------------------------------------------------------
# relmse: each path-tracing configuration at its own spp against a converged
# image (16,384 spp, FP64 accumulation of 256-spp FP32 passes)
# ---------------------------------------------------------------------------
RELMSE_CONFIGS = (  # name, scene builder, spp of the configuration, max depth
    ("cornell_256x256", lambda S: S.cornell(256, 256), 64, 8),
    ("mixed_1024x1024", lambda S: S.mixed_spheres(1024, 1024, seed=PT_SEED), 256, 16),
    ("media_512x512", lambda S: S.cornell_media(512, 512), 512, 24),
)
CONVERGED_SPP, CONVERGED_PASS = 16384, 256


def relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def run_relmse(args, world, rank, local):
    import torch

    from walkray_gb300 import scenes as S
    from walkray_gb300.api import LOW_VARIANCE, Context

    torch.cuda.set_device(local)
    ctx = Context(device=local)
    out = {}
    for name, build, spp, depth in RELMSE_CONFIGS:
        scene = build(S)
        sid = ctx.upload(scene)
        conv_spp = args.converged_spp or CONVERGED_SPP
        c0 = os.path.join(ROOT, "tests", "golden", "c0_ref.npz")
        if name == "cornell_256x256" and os.path.exists(c0):
            # configuration 0: the reference's own CPU renders (256 x 64 spp, FP64 sums)
            g = np.load(c0)
            conv = g["mean"].astype(np.float64)
            row = {"spp": spp, "max_depth": depth, "converged_spp": int(g["renders"]) * int(g["spp"]),
                   "converged": "CPU: 256 renders of WalkRay's PathTracer (64 spp each), FP64 mean (c0_ref.npz)"}
        else:
            acc = None
            t0 = time.perf_counter()
            # the low-variance estimator converges far faster to the same expectation (the
            # reference's Phong estimator has infinite variance on the mixed scene)
            for k in range(conv_spp // CONVERGED_PASS):
                img = ctx.render(sid, CONVERGED_PASS, depth, seed=7000 + k, mode="wavefront",
                                 flags=LOW_VARIANCE).astype(np.float64)
                acc = img if acc is None else acc + img
            conv = acc / (conv_spp // CONVERGED_PASS)
            row = {"spp": spp, "max_depth": depth, "converged_spp": conv_spp,
                   "converged_s": round(time.perf_counter() - t0, 2),
                   "converged": f"GPU: {conv_spp}-spp wavefront render with the low-variance estimator, FP64 sum "
                                f"of {CONVERGED_PASS}-spp passes"}
        for est, flags in (("", 0), ("_low_variance", LOW_VARIANCE)):
            for mode in ("wavefront", "megakernel"):
                ctx.render(sid, 1, depth, seed=5, mode=mode, flags=flags)  # warm
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                img = ctx.render(sid, spp, depth, seed=1, mode=mode, flags=flags).astype(np.float64)
                dt = time.perf_counter() - t0
                row[mode + est] = {"relmse": round(relmse(img, conv), 6), "seconds": round(dt, 4),
                                   "mpaths_per_s": round(img.shape[0] * img.shape[1] * spp / dt / 1e6, 2)}
        # the variance part alone: relMSE of the image against itself rendered again
        b = ctx.render(sid, spp, depth, seed=2, mode="wavefront").astype(np.float64)
        a = ctx.render(sid, spp, depth, seed=1, mode="wavefront").astype(np.float64)
        row["relmse_between_two_renders_div2"] = round(relmse(a, b) / 2, 6)
        out[name] = row
        ctx.release(sid)
    ctx.close()
    return {"metric": "relMSE at each configuration's spp vs a converged image", "value": None,
            "unit": "relMSE", "n_gpus": world, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (seeded scene generators)", "configs": out,
            "formula": "mean over pixels and channels of (I-R)^2/(R^2+1e-2); R per configuration (row 'converged'): "
                       "configuration 0 the reference's 16,384-spp CPU image, the others a 16,384-spp GPU render "
                       "with the low-variance estimator accumulated in FP64; I = one render at the configuration's spp (seed 1), with the "
                       "reference's estimator and with the low-variance one; times are wall-clock through "
                       "wr_render (host image)"}


# ---------------------------------------------------------------------------
# kd: closest-hit microbenchmark
# ---------------------------------------------------------------------------
KD_RAYS = 1 << 24


def kd_inputs(seed_rank: int):
    from walkray_gb300 import scenes as S

    s = S.icosphere_kd(8, seed=1)
    rays = S.kd_rays(s, KD_RAYS, seed=1 + seed_rank)
    return s, rays


def cpu_baseline_kd(scene, rays, sample_rays: int):
    import wr_oracle

    _, v, _, _ = scene.flatten()
    tree = wr_oracle.Tree(v, scene.global_triangles())
    sub = rays[:sample_rays]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    tree.trace(sub, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": len(sub) / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{len(sub)} of the 2^24 rays, reference traversal restated in C (oracle), "
                      f"{threads} OpenMP threads, tree build excluded"}


def run_kd(args, world, rank, local):
    import torch

    from walkray_gb300.api import Context

    torch.cuda.set_device(local)
    scene, rays = kd_inputs(rank)
    n = len(rays)
    ctx = Context(device=local, exact_traversal=args.kd_exact)
    sid = ctx.upload(scene)
    stream = torch.cuda.Stream()
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def step(i):
        ctx.trace_closest_device(sid, d_rays.data_ptr(), n, d_hits.data_ptr(), stream=stream.cuda_stream)

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step(i)
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(local) as clk:
        l0 = launches(ctx)
        ms = timed_steps(step, args.steps, stream, flush)
        n_launch = launches(ctx) - l0
    ms_max = allreduce(world, ms, "max")
    value = allreduce(world, float(n * args.steps), "sum") / (ms_max / 1e3) / 1e6
    avg_launch_s = ms / 1e3 / args.steps

    h_rays = torch.from_numpy(rays).pin_memory().numpy()
    h_hits = torch.empty((n, 4), dtype=torch.int32).pin_memory().numpy()
    ctx.trace_closest(sid, h_rays, out=h_hits)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.trace_closest(sid, h_rays, out=h_hits)
    e2e_s = allreduce(world, time.perf_counter() - t0, "max")
    e2e = allreduce(world, float(n * args.steps), "sum") / e2e_s / 1e6

    peak, peak_kind = peaks()
    achieved = KD_BYTES_PER_RAY * n / avg_launch_s / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "trace_closest_kd.json")
    if os.path.exists(prof):
        per_ray = json.load(open(prof)).get("dram_bytes_per_ray")
        traffic = round(per_ray * n, 0) if per_ray else None
    line = {
        "metric": "Mrays/s (closest hit, bit-exact vs reference)", "value": round(value, 2), "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": KD_WORKLOAD, "rays_per_step": n, "l2": "flushed (512 MiB write) before every step",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24, "d2h_bytes_per_step": n * 16},
        "roofline": {"bound": "hbm", "kernel": "k_trace_closest", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_ray": round(KD_BYTES_PER_RAY, 1)},
        "gpu_launches": int(n_launch), "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_kd(scene, rays, args.cpu_sample or (1 << 22))
    ctx.close()
    return line


def reference_kd(args):
    scene, rays = kd_inputs(0)
    vals = []
    sample = args.cpu_sample or (1 << 21)
    for _ in range(args.warmup):
        cpu_baseline_kd(scene, rays[: 1 << 16], 1 << 16)
    for k in range(args.steps):
        vals.append(cpu_baseline_kd(scene, rays[(k * sample) % len(rays):], sample))
    v = statistics.median(x["value"] for x in vals)
    cb = dict(vals[0], value=round(v, 3))
    return {"metric": "Mrays/s (closest hit, bit-exact vs reference)", "value": round(v, 3), "unit": "Mrays/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": KD_WORKLOAD, "parallelism": "host cores of rank 0",
                       "sample_per_step": f"{sample} of the 2^24 rays"},
            "cpu_baseline": cb, "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["pt", "kd", "serve", "relmse", "bpt"], default=os.environ.get("WR_BENCH_WORKLOAD", "pt"))
    ap.add_argument("--no-tune", action="store_true", help="pt: skip the wavefront autotuner (defaults instead)")
    ap.add_argument("--quick", action="store_true", help="skip the roofline profile, relMSE and CPU legs (pt)")
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--cpu-rows", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--kd-rays", type=int, default=1 << 24, help="rays per step (kd); smaller for ncu captures")
    ap.add_argument("--kd-exact", action="store_true", help="kd: visit every box the reference visits (no pruning)")
    ap.add_argument("--pt-spp", type=int, default=PT_SPP, help="samples per pixel per step (pt)")
    ap.add_argument("--mk-steps", type=int, default=5, help="timed megakernel steps beside the pt line (at most --steps)")
    ap.add_argument("--no-extras", action="store_true", help="pt: leave out the kd and serving legs")
    ap.add_argument("--pt-size", type=int, default=PT_SIZE, help="image side (pt); smaller for ncu captures")
    ap.add_argument("--serve-seconds", type=float, default=0.0,
                    help="arrival window of the request stream (0 = 60 s for --workload serve, 10 s in the pt line)")
    ap.add_argument("--serve-capacity", type=int, default=0,
                    help="serve: queue length while no request waits (wr_serve_desc.paths_in_flight; 0 = 2^22)")
    ap.add_argument("--converged-spp", type=int, default=0, help="spp of the converged image (relmse)")
    args = ap.parse_args()
    globals()["PT_SIZE"] = args.pt_size
    globals()["PT_SPP"] = args.pt_spp
    globals()["KD_RAYS"] = args.kd_rays
    world, rank, local = dist_setup()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if rank != 0:
            return
        line = {"pt": reference_pt, "kd": reference_kd, "bpt": reference_bpt}.get(args.workload, reference_pt)(args)
        print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    from walkray_gb300 import build

    build.build_lib()
    run = {"pt": run_pt, "kd": run_kd, "serve": run_serve, "relmse": run_relmse, "bpt": run_bpt}[args.workload]
    extras = args.workload == "pt" and world == 1 and not args.no_extras
    line = run(args, world, rank, local)
    if extras:
        # the kd microbenchmark and a short serving stream in the same run
        kd = run_kd(args, world, rank, local)
        line["kd"] = {k: kd[k] for k in ("metric", "value", "unit", "ms_per_step", "e2e", "roofline", "config",
                                         "gpu_launches", "clocks") if k in kd}
        if "cpu_baseline" in kd:
            line["kd"]["cpu_baseline"] = kd["cpu_baseline"]
        sv = run_serve(args, world, rank, local)
        line["serve"] = {k: sv[k] for k in sv if k not in ("n_gpus", "steps", "warmup", "higher_is_better",
                                                            "scaling", "vs_baseline", "dtype", "data")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
