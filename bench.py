"""Benchmark of the ray-cast hot path on GB300: the wavefront frame of the 155K-triangle scene.

One step = one frame at 1920x1080: primary closest hit -> shading + one any-hit shadow ray per
light -> one cosine-weighted bounce per hit (closest hit) -> shading + shadow rays -> resolve ->
TAA, replayed from a CUDA graph. The metric is rays cast per second over all passes (Mrays/s);
per-pass rates and per-frame p50/p99 latency are reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU ray-cast path for the same frame on the host cores:
the reference sources do not exist on the GPU host, so this is the oracle restatement of castRay
(pinned bit-for-bit to the reference, tests/test_oracle.py) with all host threads.
Under torchrun (N > 1) every rank renders its own frames (replicas; weak scaling) and the time is
the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s closest-/any-hit (plain vs batched/served, 1 GB300) + p50/p99 latency"
SCENE = "c2_256_2000"
RES = (1920, 1080)
SEED = 2024
CAM_DIR = (0.0, 0.8, -0.6)
CAM_UP = (0.0, 0.6, 0.8)
KERNELS = ["primary", "primary_shadow", "bounce", "bounce_shadow", "resolve_taa"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_setup(n):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
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
            self.thread.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def frame_inputs():
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300.renderer import make_lights
    s = P.standard_scene(SCENE)
    t = time.perf_counter()
    b = P.build_sbvh(s.tri_verts)
    build_s = time.perf_counter() - t
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
    return s, b, cam_pos, lights, build_s


def cpu_frame_rate(s, b, cam_pos, lights, min_seconds=8.0, max_frames=40, warm=1):
    """The oracle (castRay restatement + shading) rendering the same frames on all host threads."""
    from oracle import oracle as O
    import phantasyenginetestbed_gb300 as P
    cam = O.camera_def(cam_pos, CAM_DIR, CAM_UP, math.radians(60.0), RES)
    datas = b.slot_datas(s.datas)
    threads = O.threads()
    for f in range(warm):
        O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(f), cam_pos, SEED, f,
                       nthreads=threads)
    rays, frames, t0 = 0, 0, time.perf_counter()
    times = []
    while frames < max_frames and (time.perf_counter() - t0) < min_seconds:
        t = time.perf_counter()
        _, _, counts = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(frames),
                                      cam_pos, SEED, frames, nthreads=threads)
        times.append(time.perf_counter() - t)
        rays += int(counts.sum())
        frames += 1
    el = time.perf_counter() - t0
    return rays / el / 1e6, threads, frames, times


def run_reference(args, world, rank):
    if rank != 0:
        return
    s, b, cam_pos, lights, _ = frame_inputs()
    from oracle import oracle as O
    import phantasyenginetestbed_gb300 as P
    cam = O.camera_def(cam_pos, CAM_DIR, CAM_UP, math.radians(60.0), RES)
    datas = b.slot_datas(s.datas)
    threads = O.threads()
    for f in range(args.warmup):
        O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(f), cam_pos, SEED, f,
                       nthreads=threads)
    rays, times = 0, []
    for f in range(args.steps):
        t = time.perf_counter()
        _, _, counts = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(f),
                                      cam_pos, SEED, f, nthreads=threads)
        times.append(time.perf_counter() - t)
        rays += int(counts.sum())
    total = sum(times)
    value = rays / total / 1e6
    lat = sorted(t * 1e3 for t in times)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded heightfield + cubes scene, 155,072 triangles)",
        "config": {"workload": f"wavefront frame {RES[0]}x{RES[1]}, 1 point light, Halton jitter", "scene": SCENE,
                   "parallelism": "host threads"},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 3), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3)},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full {RES[0]}x{RES[1]} frames through the castRay restatement "
                                   "(reference sources are not on the GPU host)"},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300 import native
    from phantasyenginetestbed_gb300.renderer import READ_COLOR, CudaTracerRenderer

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    s, b, cam_pos, lights, build_s = frame_inputs()
    scene = P.Scene(b.nodes, b.verts, b.slot_datas(s.datas), s.materials)
    r = CudaTracerRenderer(use_graph=not args.no_graph)
    r.setStaticScene(scene)
    r.setTargetResolution(RES)
    r.set_seed(SEED, 0)
    r.resetTAA()
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")   # 4x the 126 MiB L2

    def frame(f):
        r.updateCamera(cam_pos, CAM_DIR, CAM_UP, 60.0, P.halton_jitter(f))
        r.render(lights, stream=stream)

    for f in range(args.warmup):
        frame(f)
    torch.cuda.synchronize()
    first = args.warmup

    # Timed region: K frames, L2 flushed before each (outside the per-frame events).
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    r.set_seed(SEED, first)
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            frame(first + k)
            ends[k].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    per = [a.elapsed_time(e) for a, e in zip(starts, ends)]
    total_ms = sum(per)
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    # Rays cast by the timed frames: the frames are deterministic, so replaying them with the same
    # seed and frame indices and reading the queue counters after each gives the exact counts.
    r.set_seed(SEED, first)
    counts = np.zeros(4, np.int64)
    for k in range(args.steps):
        frame(first + k)
        counts += r.ray_counts(stream=stream).astype(np.int64)
    rays_per_frame = int(counts.sum()) / args.steps
    value = rays_per_frame * args.steps * world / (total_ms / 1e3) / 1e6

    # Per-kernel durations (CUDA events on the render stream, direct launches) for the roofline.
    r.set_graph(False)
    r.set_kernel_timing(True)
    r.set_seed(SEED, first)
    for k in range(args.steps):
        flush.zero_()
        frame(first + k)
    torch.cuda.synchronize()
    kms, kframes = r.kernel_times()
    r.set_kernel_timing(False)
    r.set_graph(not args.no_graph)
    avg_kernel_ms = kms / max(kframes, 1)

    # End to end through the public API: parameters host -> device (pinned staging inside render),
    # frame, colour image device -> pinned host memory, every step.
    pinned = torch.empty((RES[1], RES[0], 4), dtype=torch.float32, pin_memory=True)
    host_img = pinned.numpy()
    torch.cuda.synchronize()
    r.set_seed(SEED, first)
    t0 = time.perf_counter()
    for k in range(args.steps):
        frame(first + k)
        r.read(READ_COLOR, out=host_img, stream=stream)
    e2e_s = time.perf_counter() - t0
    e2e_value = rays_per_frame * args.steps * world / e2e_s / 1e6

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    work = json.loads((ROOT / "profiles" / "work_per_ray.json").read_text())["stages"]
    io = {"primary": 48, "primary_shadow": 33, "bounce": 48, "bounce_shadow": 33}
    stage_rays = dict(zip(["primary", "primary_shadow", "bounce", "bounce_shadow"], (counts / args.steps).tolist()))
    per_kernel = {}
    for i, name in enumerate(KERNELS):
        entry = {"ms": round(float(avg_kernel_ms[i]), 4)}
        if name in stage_rays:
            n = stage_rays[name]
            w = work[name]
            bytes_per_ray = io[name] + 64 * w["n_node"] + 48 * w["n_tri"]
            entry.update({"rays": round(n, 1), "Mrays_s": round(n / (avg_kernel_ms[i] / 1e3) / 1e6, 1),
                          "alg_bytes_per_ray": round(bytes_per_ray, 1),
                          "GB_s": round(n * bytes_per_ray / (avg_kernel_ms[i] / 1e3) / 1e9, 1)})
        per_kernel[name] = entry
    dominant = max(KERNELS, key=lambda k: per_kernel[k]["ms"])
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peak = float(json.loads(peaks_path.read_text())["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    traffic = None
    tpath = ROOT / "profiles" / "ncu_traffic.json"
    if tpath.exists():
        traffic = json.loads(tpath.read_text()).get(dominant)
    dom = per_kernel[dominant]
    achieved = dom.get("GB_s")
    lat = sorted(per)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, cores, frames, _ = cpu_frame_rate(s, b, cam_pos, lights)
        cpu = {"value": round(v, 3), "unit": "Mrays/s", "cores": cores, "kind": "port",
               "sample": f"{frames} full {RES[0]}x{RES[1]} frames (~8 s) through the castRay restatement"}
    launches_per_frame = 5
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded heightfield + cubes scene, 155,072 triangles; the reference's Sponza is not in its tree)",
        "config": {"workload": f"wavefront frame {RES[0]}x{RES[1]}: primary closest -> shade + 1 any-hit shadow ray per "
                               "light -> cosine bounce closest -> shade + shadow -> resolve + TAA",
                   "scene": SCENE, "triangles": int(len(s.tri_verts)), "bvh_nodes": int(len(b.nodes)),
                   "bvh_slots": int(len(b.verts)), "sbvh_build_s": round(build_s, 2), "lights": 1,
                   "rays_per_frame": round(rays_per_frame, 1), "rays_by_pass": {k: round(v, 1) for k, v in stage_rays.items()},
                   "cuda_graph": not args.no_graph, "l2": "flushed before every timed frame (512 MiB write)",
                   "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 4), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 4)},
        "passes": per_kernel,
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4) if achieved else None, "traffic": traffic,
                     "peak_source": peak_src,
                     "note": "algorithmic bytes = ray I/O + 64 B x nodes + 48 B x triangle tests per ray (oracle "
                             "castDebugRay means, profiles/work_per_ray.json); most of it is served from L1/L2"},
        "clocks": clocks.summary(),
        "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s",
                "h2d_bytes_per_step": int(native.lib().phe_renderer_frame_param_bytes()),
                "d2h_bytes_per_step": RES[0] * RES[1] * 16},
        "gpu_launches": launches_per_frame * args.steps,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
