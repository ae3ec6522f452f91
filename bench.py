#!/usr/bin/env python3
"""Benchmark driver.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload kd|pt]

Prints ONE JSON line (rank 0).  Workloads:

  pt  (default) wavefront path tracing of the mixed-material scene: 25
      displaced level-5 icospheres (512,006 triangles) on a ground plane,
      1024x1024, max depth 16; one step = one sample per pixel (1,048,576
      paths).  Metric Mpaths/s.
  kd  closest-hit microbenchmark: level-8 displaced icosphere (1,310,720
      triangles), 2^24 rays; one step = all rays.  Metric Mrays/s.

`value` is device-timed with CUDA events per step on the launching stream,
L2 flushed (a 512 MiB write) before every step, inputs resident in HBM;
`e2e` runs the same steps through the public C ABI with host buffers
(pinned), host<->device copies inside the timed region.  `--impl reference`
times WalkRay's CPU algorithm (the oracle restatement, all host threads) on
a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
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
# algorithmic bytes: ray in (24) + hit out (16) + per box test 8 B topology
# + 24 B AABB + per triangle test 3 x 16 B vertices + 4 B object id
KD_BYTES_PER_RAY = 24 + 16 + KD_BOX_TESTS * 32 + KD_TRI_TESTS * 52


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


def allmax(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# kd: closest-hit microbenchmark
# ---------------------------------------------------------------------------
def kd_inputs(seed_rank: int):
    from walkray_gb300 import scenes as S

    s = S.icosphere_kd(8, seed=1)
    rays = S.kd_rays(s, 1 << 24, seed=1 + seed_rank)
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
    ctx = Context(device=local)
    sid = ctx.upload(scene)
    stream = torch.cuda.Stream()
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def step():
        ctx.trace_closest_device(sid, d_rays.data_ptr(), n, d_hits.data_ptr(), stream=stream.cuda_stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    barrier(world)
    evs = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t_wall = time.perf_counter()
        with torch.cuda.stream(stream):
            for _ in range(args.steps):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                step()
                b.record(stream)
                evs.append((a, b))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    ms = sum(a.elapsed_time(b) for a, b in evs)
    ms_max = allmax(world, ms)
    units = allsum(world, float(n * args.steps))
    value = units / (ms_max / 1e3) / 1e6
    avg_launch_s = ms / 1e3 / args.steps

    # e2e through the host-buffer entry point, pinned host memory
    h_rays = torch.from_numpy(rays).pin_memory().numpy()
    h_hits = torch.empty((n, 4), dtype=torch.int32).pin_memory().numpy()
    ctx.trace_closest(sid, h_rays, out=h_hits)  # warm
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.trace_closest(sid, h_rays, out=h_hits)
    e2e_s = allmax(world, time.perf_counter() - t0)
    e2e = allsum(world, float(n * args.steps)) / e2e_s / 1e6

    peak, peak_kind = peaks()
    achieved = KD_BYTES_PER_RAY * n / avg_launch_s / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "trace_closest_kd.json")
    if os.path.exists(prof):
        traffic = json.load(open(prof)).get("dram_bytes_per_ray")
        traffic = traffic * n if traffic else None
    line = {
        "metric": "Mrays/s (closest hit, bit-exact vs reference)", "value": round(value, 2), "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "kd: level-8 displaced icosphere (1,310,720 tris), 2^24 rays (origins in 2x bounds, "
                               "uniform directions)", "rays_per_step": n, "l2": "flushed (512 MiB write) before every step",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24, "d2h_bytes_per_step": n * 16},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_ray": round(KD_BYTES_PER_RAY, 1)},
        "gpu_launches": args.steps, "clocks": clk.summary(),
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
            "impl": "reference", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": "kd: level-8 displaced icosphere (1,310,720 tris), 2^24 rays",
                       "rays_per_step": sample},
            "cpu_baseline": cb, "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["kd", "pt"], default=os.environ.get("WR_BENCH_WORKLOAD", "kd"))
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if rank != 0:
            return
        line = reference_kd(args)
        print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    from walkray_gb300 import build

    build.build_lib()
    line = run_kd(args, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
