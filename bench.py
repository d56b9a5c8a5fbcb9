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
REF_BUDGET_S = 90.0   # host seconds the reference arm spends in its timed steps
SEED = 2024
CAM_DIR = (0.0, 0.8, -0.6)
CAM_UP = (0.0, 0.6, 0.8)
KERNELS = ["primary_trace", "primary_shade", "primary_shadow", "bounce_bin", "bounce_trace", "bounce_shade",
           "bounce_shadow", "resolve_taa"]
KERNELS_FUSED = ["primary", "primary_shadow", "bounce_bin", "bounce", "bounce_shadow", "resolve_taa"]
# traversal kernel -> the pass whose rays it casts
TRACE_PASS = {"primary_trace": "primary", "primary": "primary", "primary_shadow": "primary_shadow",
              "bounce_trace": "bounce", "bounce": "bounce", "bounce_shadow": "bounce_shadow"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000,
                    help="frames timed (default: about one second of frames, so the clock sampler sees the load)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--pipeline", choices=["fused", "split"], default="fused",
                    help="fused: traversal + shading in one kernel per bounce (4 kernels with merged shadows); split: 7 kernels")
    ap.add_argument("--refill", type=int, default=28, help="lane-refill threshold of the split pipeline")
    ap.add_argument("--sort-window", type=int, default=0, help="bin bounce rays by octant in windows of N (0 = off)")
    ap.add_argument("--shadows", choices=["merged", "beside", "in-order"], default="merged",
                    help="shadow-pass schedule: one pass over both queues after the bounce pass (default), the "
                         "primary shadow pass beside the bounce pass, or each after its own pass")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["frame", "plain", "batch", "large", "serve", "sizes"], default="frame",
                    help="frame (default, the headline): 1080p wavefront frame; batch: 64 uneven batches over 4 "
                         "scenes in one launch vs 64 plain launches; large: 8.6M-triangle scene, 4096x4096, 4 "
                         "lights; serve: Poisson request arrivals through the serving loop; sizes: launch time "
                         "against rays per launch (16K..16M) for each ray-cast entry point")
    ap.add_argument("--res", type=int, default=4096, help="large: width and height of the frame")
    ap.add_argument("--rates", default="200,500,1000", help="serve: arrival rates (requests/s)")
    ap.add_argument("--duration", type=float, default=2.0, help="serve: seconds of arrivals per rate")
    ap.add_argument("--render-slots", type=int, default=8, help="serve: concurrent render requests")
    ap.add_argument("--batch-window-us", type=int, default=0, help="serve: wave batching window")
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


def aggregate_over_ranks(rays_this_rank: float, ms_this_rank: float, dist=None, device=None):
    """Whole-job throughput of replicas: rays summed over ranks / the slowest rank's time (ms).
    Returns (total rays, max ms, Mrays/s)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return rays_this_rank, ms_this_rank, rays_this_rank / (ms_this_rank / 1e3) / 1e6
    import torch
    t = torch.tensor([float(rays_this_rank), float(ms_this_rank)], dtype=torch.float64, device=device)
    rays = t[:1].clone()
    ms = t[1:].clone()
    dist.all_reduce(rays, op=dist.ReduceOp.SUM)
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    r, m = float(rays.item()), float(ms.item())
    return r, m, r / (m / 1e3) / 1e6


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


FRAME_WORKLOAD = (f"wavefront frame {RES[0]}x{RES[1]}: primary closest -> shade + 1 any-hit shadow ray per light -> "
                  "cosine bounce closest -> shade + shadow -> resolve + TAA")
FRAME_DATA = "synthetic (seeded heightfield + cubes scene, 155,072 triangles; the reference's Sponza is not in its tree)"


def frame_config(s, b, build_s) -> dict:
    """The frame workload's identifying keys, the same in both arms."""
    return {"workload": FRAME_WORKLOAD, "scene": SCENE, "triangles": int(len(s.tri_verts)),
            "bvh_nodes": int(len(b.nodes)), "bvh_slots": int(len(b.verts)), "sbvh_build_s": round(build_s, 2),
            "lights": 1}


def run_reference(args, world, rank):
    if rank != 0:
        return
    s, b, cam_pos, lights, build_s = frame_inputs()
    from oracle import oracle as O
    import phantasyenginetestbed_gb300 as P
    cam = O.camera_def(cam_pos, CAM_DIR, CAM_UP, math.radians(60.0), RES)
    datas = b.slot_datas(s.datas)
    threads = O.threads()
    full = []
    for f in range(max(1, args.warmup)):
        t = time.perf_counter()
        O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(f), cam_pos, SEED, f,
                       nthreads=threads)
        full.append(time.perf_counter() - t)
    # Each step renders a band of rows sized so that all steps take about REF_BUDGET_S (whole frames
    # when the steps are few); the band moves down the frame from step to step.
    rows = max(8, min(RES[1], int(RES[1] * (REF_BUDGET_S / args.steps) / min(full))))
    rays, times = 0, []
    for f in range(args.steps):
        r0 = (f * rows) % RES[1]
        band = (r0, min(RES[1], r0 + rows))
        t = time.perf_counter()
        _, _, counts = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(f),
                                      cam_pos, SEED, f, nthreads=threads, rows=band)
        times.append(time.perf_counter() - t)
        rays += int(counts.sum())
    total = sum(times)
    value = rays / total / 1e6
    lat = sorted(t * 1e3 for t in times)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": FRAME_DATA,
        "config": {**frame_config(s, b, build_s), "parallelism": f"host threads x{threads}"},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 3), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3)},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": (f"{args.steps} frames of the {RES[0]}x{RES[1]} workload through the castRay "
                                    f"restatement, a band of up to {rows} rows of each (moving down the frame; whole "
                                    f"frames take {min(full):.2f} s here); the reference sources are not on "
                                    "the GPU host")},
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
    r.set_pipeline(fused=args.pipeline == "fused", refill=args.refill, sort_window=args.sort_window)
    r.set_shadow_schedule({"in-order": 0, "beside": 1, "merged": 2}[args.shadows])
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
    # Rays cast by the timed frames: the frames are deterministic, so replaying them with the same
    # seed and frame indices and reading the queue counters after each gives the exact counts.
    r.set_seed(SEED, first)
    counts = np.zeros(4, np.int64)
    for k in range(args.steps):
        frame(first + k)
        counts += r.ray_counts(stream=stream).astype(np.int64)
    rays_per_frame = int(counts.sum()) / args.steps
    _, total_ms, value = aggregate_over_ranks(rays_per_frame * args.steps, total_ms, dist,
                                              torch.device("cuda", local) if dist else None)

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
    # frame, colour image device -> pinned host memory, every step. Pipelined: each frame's image is
    # read back asynchronously into one of two pinned host images while the next frame renders (the
    # way a real-time host consumes frames); the clock stops once the last image is in host memory.
    # Blocking: the synchronous read after every frame.
    host_imgs = [torch.empty((RES[1], RES[0], 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    torch.cuda.synchronize()
    r.set_seed(SEED, first)
    t0 = time.perf_counter()
    for k in range(args.steps):
        frame(first + k)
        r.read_async(host_imgs[k & 1], READ_COLOR, stream=stream)
    r.read_wait()
    e2e_s = time.perf_counter() - t0
    e2e_value = rays_per_frame * args.steps * world / e2e_s / 1e6
    torch.cuda.synchronize()
    r.set_seed(SEED, first)
    t0 = time.perf_counter()
    for k in range(args.steps):
        frame(first + k)
        r.read(READ_COLOR, out=host_imgs[0], stream=stream)
    e2e_blocking = rays_per_frame * args.steps * world / (time.perf_counter() - t0) / 1e6

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    work = json.loads((ROOT / "profiles" / "work_per_ray.json").read_text())["stages"]
    io = {"primary": 48, "primary_shadow": 33, "bounce": 48, "bounce_shadow": 33}
    stage_rays = dict(zip(["primary", "primary_shadow", "bounce", "bounce_shadow"], (counts / args.steps).tolist()))
    per_kernel = {}
    names = KERNELS_FUSED if args.pipeline == "fused" else KERNELS
    if args.pipeline == "fused" and args.shadows == "merged":
        names = ["primary", "bounce_bin", "bounce", "shadows", "resolve_taa"]
    if args.sort_window == 0:
        names = [k for k in names if k != "bounce_bin"]

    def pass_bytes(pas):
        w = work[pas]
        return io[pas] + 64 * w["n_node"] + 48 * w["n_tri"]

    for i, name in enumerate(names):
        entry = {"ms": round(float(avg_kernel_ms[i]), 4)}
        if name == "shadows":   # both shadow queues in one launch
            n = stage_rays["primary_shadow"] + stage_rays["bounce_shadow"]
            bytes_per_ray = (stage_rays["primary_shadow"] * pass_bytes("primary_shadow") +
                             stage_rays["bounce_shadow"] * pass_bytes("bounce_shadow")) / n
            entry.update({"rays": round(n, 1), "Mrays_s": round(n / (avg_kernel_ms[i] / 1e3) / 1e6, 1),
                          "alg_bytes_per_ray": round(bytes_per_ray, 1),
                          "GB_s": round(n * bytes_per_ray / (avg_kernel_ms[i] / 1e3) / 1e9, 1)})
        elif name in TRACE_PASS:
            pas = TRACE_PASS[name]
            n = stage_rays[pas]
            bytes_per_ray = pass_bytes(pas)
            entry.update({"rays": round(n, 1), "Mrays_s": round(n / (avg_kernel_ms[i] / 1e3) / 1e6, 1),
                          "alg_bytes_per_ray": round(bytes_per_ray, 1),
                          "GB_s": round(n * bytes_per_ray / (avg_kernel_ms[i] / 1e3) / 1e9, 1)})
        per_kernel[name] = entry
    dominant = max((k for k in names if "rays" in per_kernel[k]), key=lambda k: per_kernel[k]["ms"])
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peak = float(json.loads(peaks_path.read_text())["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    traffic, issue = None, None
    tpath = ROOT / "profiles" / "ncu_traffic.json"
    if tpath.exists():
        nc = json.loads(tpath.read_text())
        traffic = nc.get(dominant)
        if f"{dominant}_inst_per_cycle" in nc:
            # the limit that binds (the scene is L2-resident): issue, from the committed ncu capture
            issue = {"inst_per_cycle": nc[f"{dominant}_inst_per_cycle"], "of": 4,
                     "frac": round(nc[f"{dominant}_inst_per_cycle"] / 4, 3),
                     "simd_efficiency": nc.get(f"{dominant}_simd_efficiency"),
                     "dram_frac": nc.get(f"{dominant}_dram_throughput"),
                     "l2_frac": nc.get(f"{dominant}_l2_throughput"), "l1_frac": nc.get(f"{dominant}_l1_throughput"),
                     "l2_bytes": nc.get(f"{dominant}_l2_bytes"), "source": "profiles/bounce_kernel_1080p_ncu.md"}
    dom = per_kernel[dominant]
    achieved = dom.get("GB_s")
    lat = sorted(per)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, cores, frames, _ = cpu_frame_rate(s, b, cam_pos, lights)
        cpu = {"value": round(v, 3), "unit": "Mrays/s", "cores": cores, "kind": "port",
               "sample": f"{frames} full {RES[0]}x{RES[1]} frames (~8 s) through the castRay restatement"}
    launches_per_frame = len(names)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": FRAME_DATA,
        "config": {**frame_config(s, b, build_s),
                   "rays_per_frame": round(rays_per_frame, 1), "rays_by_pass": {k: round(v, 1) for k, v in stage_rays.items()},
                   "cuda_graph": not args.no_graph, "pipeline": args.pipeline,
                   "refill_threshold": args.refill, "sort_window": args.sort_window,
                   "shadow_schedule": args.shadows if args.pipeline == "fused" else "in-order", "l2": "flushed before every timed frame (512 MiB write)",
                   "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 4), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 4)},
        "passes": per_kernel,
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4) if achieved else None, "traffic": traffic,
                     "peak_source": peak_src, "issue": issue,
                     "note": "algorithmic bytes = ray I/O + 64 B x nodes + 48 B x triangle tests per ray (oracle "
                             "castDebugRay means, profiles/work_per_ray.json); the scene is L2-resident, so most of "
                             "it is served from L1/L2 (traffic = DRAM bytes per launch) and frac is an effective "
                             "bandwidth; the binding limit is instruction issue (see issue)"},
        "clocks": clocks.summary(),
        "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s",
                "h2d_bytes_per_step": int(native.lib().phe_renderer_frame_param_bytes()),
                "d2h_bytes_per_step": RES[0] * RES[1] * 16,
                "mode": "pipelined: colour image read back asynchronously (two pinned host images) while the "
                        "next frame renders; clock stops when the last image is in host memory",
                "blocking_value": round(e2e_blocking, 2)},
        "gpu_launches": launches_per_frame * args.steps,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------------------------
# Additional workloads (not the headline line): uneven batches, large incoherent scene, serving.
# ---------------------------------------------------------------------------------------------

def _scene_with_bvh(name):
    import phantasyenginetestbed_gb300 as P
    s = P.standard_scene(name)
    t = time.perf_counter()
    b = P.build_sbvh(s.tri_verts)
    return s, b, time.perf_counter() - t


def _surface_rays(s, n, rng, tmax=3.4028235e38):
    """Rays from random points on random triangles in uniformly random directions."""
    import phantasyenginetestbed_gb300 as P
    tri = s.tri_verts[rng.integers(0, len(s.tri_verts), n)]
    a, b2 = rng.random((n, 1), np.float32), rng.random((n, 1), np.float32)
    flip = (a + b2) > 1
    a = np.where(flip, 1 - a, a)
    b2 = np.where(flip, 1 - b2, b2)
    p = tri[:, 0:3] + a * (tri[:, 3:6] - tri[:, 0:3]) + b2 * (tri[:, 6:9] - tri[:, 0:3])
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, P.RAY_IN_DTYPE)
    rays["origin"] = p
    rays["dir"] = d
    rays["tMin"] = np.float32(1e-3)
    rays["tMax"] = np.float32(tmax)
    return rays


def _percentiles(times_ms):
    """p50 / p99 of per-step times (ms): the time for the whole 64-batch mix to complete."""
    t = sorted(times_ms)
    return {"p50": round(t[len(t) // 2], 4), "p99": round(t[min(len(t) - 1, int(0.99 * len(t)))], 4)}


def _timed(fn, steps, stream, flush=None):
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        if flush is not None:
            flush.zero_()
        ev[k][0].record(stream)
        fn()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def run_plain(args):
    """The plain closest-hit configuration: 512x512 pinhole primary rays on the 9,392-triangle scene
    (64x64-cell heightfield + 100 axis-aligned cubes), through phe_cast_closest (persistent),
    phe_cast_closest_plain (one ray per thread) and phe_cast_any, with the CPU castRay restatement on
    all host cores beside it. Each step is one launch over all rays; L2 flushed before each."""
    import torch
    import phantasyenginetestbed_gb300 as P
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    s, b, build_s = _scene_with_bvh("c1_64_100")
    scene = P.Scene(b.nodes, b.verts)
    res = (512, 512)
    n = res[0] * res[1]
    cam = P.camera_def((0.5, -0.3, 0.6), CAM_DIR, CAM_UP, 60.0, res)
    rays = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    P.gen_primary_rays(rays, cam, res, order=1)
    hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    vis = torch.empty(n, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    out = {}
    for layout, lname in ((0, "binary"), (1, "wide4")):
        scene.set_layout(layout)
        for name, fn in (("closest_persistent", lambda: P.cast_closest(scene, rays, hits, n, stream=stream)),
                         ("closest_plain", lambda: P.cast_closest_plain(scene, rays, hits, n, stream=stream)),
                         ("any", lambda: P.cast_any(scene, rays, vis, n, stream=stream))):
            for _ in range(args.warmup):
                fn()
            t = statistics.median(_timed(fn, args.steps, stream, flush))
            out[f"{name}_{lname}"] = {"ms": round(t, 4), "Mrays_s": round(n / t / 1e3, 1)}
    scene.set_layout(0)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        host_rays = rays.cpu().numpy().view(P.RAY_IN_DTYPE)
        O.cast_rays(b.nodes, b.verts, host_rays)
        t0, reps = time.perf_counter(), 0
        while time.perf_counter() - t0 < 5.0:
            O.cast_rays(b.nodes, b.verts, host_rays)
            reps += 1
        el = time.perf_counter() - t0
        cpu = {"value": round(n * reps / el / 1e6, 2), "unit": "Mrays/s", "cores": O.threads(), "kind": "port",
               "sample": f"{reps} passes over the 512x512 primary rays (~5 s)"}
    line = {"workload": "plain", "metric": METRIC, "unit": "Mrays/s", "rays": n, "triangles": int(len(s.tri_verts)),
            "bvh_nodes": int(len(b.nodes)), "bvh_slots": int(len(b.verts)), "launches": out, "cpu_baseline": cpu,
            "l2": "flushed before every timed launch"}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """64 ray batches of uneven size (log-uniform 1K..1M), 50% pinhole / 50% random-surface rays, over 4
    resident scenes (10K/155K/1M/2M triangles), 70/30 closest/any: one autotuned persistent launch
    replayed from a CUDA graph vs 64 plain launches (and vs 64 launches each followed by a device
    synchronisation, as the reference's launchers do)."""
    import torch
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300.batch import ANY, CLOSEST, Batch, save_tuning
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    names = ["c3_10k", "c3_155k", "c3_1m", "c3_2m"]
    built = [_scene_with_bvh(n) for n in names]
    scenes = [P.Scene(b.nodes, b.verts) for _, b, _ in built]
    rng = np.random.default_rng(2024)
    items, total = [], 0
    for i in range(64):
        n = int(np.exp(rng.uniform(np.log(1024), np.log(1 << 20))))
        si = int(rng.integers(0, 4))
        kind = CLOSEST if rng.random() < 0.7 else ANY
        s = built[si][0]
        d_rays = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
        if i % 2 == 0:
            k = s.scale
            w = 1024
            h = (n + w - 1) // w
            cam = P.camera_def((0.5 * k, -0.3 * k, 0.6 * k), CAM_DIR, CAM_UP, 60.0, (w, h))
            full = torch.empty(w * h * 32, dtype=torch.uint8, device="cuda")
            P.gen_primary_rays(full, cam, (w, h), order=0)
            d_rays.copy_(full[: n * 32])
        else:
            d_rays.copy_(torch.from_numpy(_surface_rays(s, n, rng).view(np.uint8)))
        out = torch.empty(n * (16 if kind == CLOSEST else 1), dtype=torch.uint8, device="cuda")
        items.append((si, kind, n, d_rays, out))
        total += n
    torch.cuda.synchronize()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    batch = Batch(scenes, items, use_graph=False)
    best, best_ms, table = batch.autotune(repeats=3)
    save_tuning(ROOT / "profiles" / "batch_autotune.json", best, best_ms, table,
                command=f"python bench.py --workload batch --steps {args.steps} --warmup {args.warmup} "
                        "(phe_batch_autotune, repeats=3, cold L2)")
    batch.set_params(block_size=best["blockSize"], blocks_per_sm=best["blocksPerSM"], order=best["order"], use_graph=True,
                     layout=best["layout"], stack_shared=best["stackShared"], sort_window=best["sortWindow"])
    for _ in range(args.warmup):
        batch.launch(stream)
    t_batched = _timed(lambda: batch.launch(stream), args.steps, stream, flush)

    def plain():
        for si, kind, n, d_rays, out in items:
            (P.cast_closest if kind == CLOSEST else P.cast_any)(scenes[si], d_rays, out, n, stream=stream)

    def plain_sync():
        for si, kind, n, d_rays, out in items:
            (P.cast_closest if kind == CLOSEST else P.cast_any)(scenes[si], d_rays, out, n, stream=stream)
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        plain()
    t_plain = _timed(plain, args.steps, stream, flush)
    steps_sync = max(3, args.steps // 5)
    # wall clock of the synchronised variant (host waits are part of that launch model)
    walls = []
    for _ in range(steps_sync):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        plain_sync()
        walls.append((time.perf_counter() - t) * 1e3)
    mb = statistics.median(t_batched)
    mp = statistics.median(t_plain)
    ms_sync = statistics.median(walls)
    line = {"workload": "batch", "metric": METRIC, "unit": "Mrays/s", "batches": 64, "rays": total,
            "scenes": {n: int(len(b.verts)) for n, (_, b, _) in zip(names, built)},
            "batched_graph": {"ms": round(mb, 4), "Mrays_s": round(total / mb / 1e3, 1), "params": best,
                              "latency_ms": _percentiles(t_batched)},
            "plain_64_launches": {"ms": round(mp, 4), "Mrays_s": round(total / mp / 1e3, 1),
                                  "latency_ms": _percentiles(t_plain)},
            "plain_64_launches_synchronised": {"ms": round(ms_sync, 4), "Mrays_s": round(total / ms_sync / 1e3, 1),
                                               "latency_ms": _percentiles(walls)},
            "speedup_vs_plain": round(mp / mb, 3), "speedup_vs_synchronised": round(ms_sync / mb, 3),
            "autotune_candidates": len(table), "layouts_tried": sorted({r["layout"] for r in table}),
            "l2": "flushed before every timed step"}
    print(json.dumps(line), flush=True)


def run_sizes(args):
    """Launch time against batch size on the 155,072-triangle scene: 16K..16M rays per launch through
    phe_cast_closest (persistent warps), phe_cast_closest_plain (one ray per thread) and phe_cast_any,
    for coherent rays (a 4096x4096 pinhole camera, 8x8-tile order) and incoherent rays (uniform origins
    above the terrain, uniform directions, seeded). L2 flushed before each timed launch; median of
    args.steps launches."""
    import torch
    import phantasyenginetestbed_gb300 as P
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    s, b, _ = _scene_with_bvh("c2_256_2000")
    scene = P.Scene(b.nodes, b.verts)
    k = s.scale
    res = (4096, 4096)
    N = res[0] * res[1]
    coherent = torch.empty(N * 32, dtype=torch.uint8, device="cuda")
    P.gen_primary_rays(coherent, P.camera_def((0.5 * k, -0.3 * k, 0.6 * k), CAM_DIR, CAM_UP, 60.0, res), res, order=1)
    rng = np.random.default_rng(SEED)
    inc = np.zeros(N, P.RAY_IN_DTYPE)
    inc["origin"] = rng.uniform([0, 0, 0.02 * k], [k, k, 0.3 * k], (N, 3)).astype(np.float32)
    d = rng.normal(size=(N, 3))
    inc["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    inc["tMin"], inc["tMax"] = np.float32(1e-4), np.float32(3.4028235e38)
    incoherent = torch.from_numpy(inc.view(np.uint8)).cuda()
    hits = torch.empty(N * 16, dtype=torch.uint8, device="cuda")
    vis = torch.empty(N, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    out = {}
    for rname, rays in (("coherent", coherent), ("incoherent", incoherent)):
        for n in (1 << 14, 1 << 16, 1 << 18, 1 << 20, 1 << 22, 1 << 24):
            row = {}
            for name, fn in (("closest_persistent", lambda: P.cast_closest(scene, rays, hits, n, stream=stream)),
                             ("closest_plain", lambda: P.cast_closest_plain(scene, rays, hits, n, stream=stream)),
                             ("any", lambda: P.cast_any(scene, rays, vis, n, stream=stream))):
                for _ in range(args.warmup):
                    fn()
                t = statistics.median(_timed(fn, args.steps, stream, flush))
                row[name] = {"ms": round(t, 4), "Mrays_s": round(n / t / 1e3, 1)}
            out[f"{rname}_{n}"] = row
    line = {"workload": "sizes", "metric": METRIC, "unit": "Mrays/s", "triangles": int(len(s.tri_verts)),
            "launches": out, "l2": "flushed before every timed launch"}
    print(json.dumps(line), flush=True)


def run_large(args):
    """8.63M-triangle scene (2048x2048-cell heightfield + 20,000 cubes, world x32), 4096x4096 frame with
    4 point lights: 16.8M primary rays, ~16M bounce rays (cosine-weighted), shadow rays to 4 lights."""
    import torch
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300.renderer import CudaTracerRenderer, make_lights
    torch.cuda.set_device(0)
    res = (args.res, args.res)
    s, b, build_s = _scene_with_bvh("c4_2048_20000")
    scene = P.Scene(b.nodes, b.verts, b.slot_datas(s.datas), s.materials)
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    lights = make_lights(np.array([[0.5, 0.5, 2.0], [0.1, 0.1, 1.0], [0.9, 0.2, 1.5], [0.3, 0.9, 0.8]], np.float32)
                         * np.float32(k), range_=1000.0 * k)
    r = CudaTracerRenderer(use_graph=True)
    r.setStaticScene(scene)
    r.setTargetResolution(res)
    stream = torch.cuda.current_stream()
    r.set_seed(SEED, 0)
    for f in range(args.warmup):
        r.updateCamera(cam_pos, CAM_DIR, CAM_UP, 60.0, P.halton_jitter(f))
        r.render(lights, stream=stream)
    steps = max(3, min(args.steps, 10))
    r.set_graph(False)
    r.set_kernel_timing(True)
    r.set_seed(SEED, args.warmup)
    counts = np.zeros(4, np.int64)
    walls = []
    for f in range(steps):
        r.updateCamera(cam_pos, CAM_DIR, CAM_UP, 60.0, P.halton_jitter(f))
        r.render(lights, stream=stream)
        counts += r.ray_counts(stream=stream).astype(np.int64)
    kms, frames = r.kernel_times()
    avg = kms / frames
    counts = counts / steps
    frame_ms = float(avg.sum())
    names = ["primary", "bounce", "shadows", "resolve_taa"]   # the default (merged) shadow schedule
    passes = {}
    for i, nm in enumerate(names):
        e = {"ms": round(float(avg[i]), 3)}
        if nm == "shadows":
            n = counts[1] + counts[3]
            e.update({"rays": int(n), "Mrays_s": round(n / avg[i] / 1e3, 1),
                      "primary_shadow_rays": int(counts[1]), "bounce_shadow_rays": int(counts[3])})
        elif nm in TRACE_PASS:
            n = counts[["primary", "primary_shadow", "bounce", "bounce_shadow"].index(TRACE_PASS[nm])]
            e.update({"rays": int(n), "Mrays_s": round(n / avg[i] / 1e3, 1)})
        passes[nm] = e
    line = {"workload": "large", "metric": METRIC, "unit": "Mrays/s", "triangles": int(len(s.tri_verts)),
            "bvh_nodes": int(len(b.nodes)), "bvh_slots": int(len(b.verts)), "sbvh_build_s": round(build_s, 1),
            "scene_bytes": scene.device_bytes(), "res": res, "lights": 4, "frame_ms": round(frame_ms, 3),
            "rays_per_frame": int(counts.sum()), "value": round(counts.sum() / frame_ms / 1e3, 1), "passes": passes}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Poisson arrivals of render requests (256x256..1920x1080 log-uniform, 1-4 spp) and ray-query
    requests (4K..512K rays log-uniform, 70/30 closest/any) against 8 resident scenes of 50K..4M
    triangles, under a 120 GB budget, through the continuous-batching server and the serial baseline."""
    import threading as th
    import torch
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300.renderer import make_lights
    from phantasyenginetestbed_gb300.serve import REQ_ANY, REQ_CLOSEST, Server, pinned
    torch.cuda.set_device(0)
    grids = [160, 256, 362, 512, 724, 1024, 1240, 1448]
    built, scenes = [], []
    t0 = time.perf_counter()
    for i, g in enumerate(grids):
        s = P.generate_scene(g, 100, False, 500 + i)
        b = P.build_sbvh(s.tri_verts)
        built.append((s, b))
        scenes.append(P.Scene(b.nodes, b.verts, b.slot_datas(s.datas), s.materials))
    build_s = time.perf_counter() - t0
    rng = np.random.default_rng(7)
    pools = []
    for s, _ in built:
        rp = pinned(1 << 19, P.RAY_IN_DTYPE)
        rp[:] = _surface_rays(s, 1 << 19, rng)
        pools.append(rp)
    out_ring = [pinned((1 << 19) * 16, np.uint8) for _ in range(8)]
    img_ring = [pinned((1080, 1920, 4), np.float32) for _ in range(8)]

    def make_requests(rate, duration, seed):
        r = np.random.default_rng(seed)
        t, reqs = 0.0, []
        while True:
            t += r.exponential(1.0 / rate)
            if t > duration:
                break
            si = int(r.integers(0, len(scenes)))
            if r.random() < 0.5:
                pix = np.exp(r.uniform(np.log(256 * 256), np.log(1920 * 1080)))
                w = int(min(1920, max(256, round(np.sqrt(pix * 16 / 9) / 8) * 8)))
                h = int(max(256 // 2, round(pix / w / 8) * 8))
                h = min(h, (1920 * 1080) // w // 8 * 8)
                reqs.append((t, "render", si, (w, h), int(r.integers(1, 5))))
            else:
                n = int(np.exp(r.uniform(np.log(4096), np.log(1 << 19))))
                reqs.append((t, "rays", si, n, REQ_CLOSEST if r.random() < 0.7 else REQ_ANY))
        return reqs

    def run(server, ids, reqs, burst=False):
        cams = {}
        start = time.perf_counter() + 0.05
        sub = []
        for j, q in enumerate(reqs):
            dt = start + q[0] - time.perf_counter()
            if dt > 0 and not burst:
                time.sleep(dt)
            arrival = (start + q[0])
            if q[1] == "render":
                s, _ = built[q[2]]
                k = s.scale
                cp = (0.5 * k, -0.3 * k, 0.6 * k)
                key = (q[2], q[3])
                if key not in cams:
                    cams[key] = P.camera_def(cp, CAM_DIR, CAM_UP, 60.0, q[3])
                lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
                rid = server.submit_render(ids[q[2]], q[3], q[4], cams[key], cp, lights, 11 + j, img_ring[j % 8])
            else:
                rid = server.submit_rays(ids[q[2]], pools[q[2]][: q[3]], out_ring[j % 8], q[4])
            sub.append((rid, arrival))
        server.drain()
        lat, rays, t_first, t_last, errors = [], 0, None, 0.0, 0
        for rid, arrival in sub:
            st = server.poll(rid)
            errors += st.status != 0
            lat.append(st.doneMs - st.submitMs)
            rays += st.rays
            t_last = max(t_last, st.doneMs)
            t_first = st.submitMs if t_first is None else min(t_first, st.submitMs)
            server.release(rid)
        lat.sort()
        span_ms = t_last - t_first
        return {"requests": len(sub), "errors": int(errors), "p50_ms": round(lat[len(lat) // 2], 3),
                "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3),
                "rays": int(rays), "span_s": round(span_ms / 1e3, 3), "Mrays_s": round(rays / span_ms / 1e3, 1)}

    results = {}
    for rate in [float(x) for x in args.rates.split(",")]:
        reqs = make_requests(rate, args.duration, int(rate))
        row = {}
        for mode in ("continuous", "serial"):
            server = Server(memory_budget=120 << 30, render_slots=args.render_slots, serial=(mode == "serial"),
                            batch_window_us=args.batch_window_us)
            ids = [server.add_scene(sc) for sc in scenes]
            row[mode] = run(server, ids, reqs)
            server.close()
        results[str(int(rate))] = row
    # Saturation: the highest rate's requests all submitted at once (makespan throughput).
    burst = {}
    reqs = make_requests(max(float(x) for x in args.rates.split(",")), args.duration, 99)
    for mode in ("continuous", "serial"):
        server = Server(memory_budget=120 << 30, render_slots=args.render_slots, serial=(mode == "serial"),
                        batch_window_us=args.batch_window_us)
        ids = [server.add_scene(sc) for sc in scenes]
        burst[mode] = run(server, ids, reqs, burst=True)
        server.close()
    burst["speedup"] = round(burst["continuous"]["Mrays_s"] / max(burst["serial"]["Mrays_s"], 1e-9), 3)
    results["burst"] = burst
    line = {"workload": "serve", "metric": METRIC, "unit": "Mrays/s",
            "scenes_triangles": [int(len(s.tri_verts)) for s, _ in built], "scene_build_s": round(build_s, 1),
            "budget_bytes": 120 << 30, "arrivals_s": args.duration, "render_slots": args.render_slots,
            "batch_window_us": args.batch_window_us, "rates": results}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "frame":
        run_ours(args, world, rank, local)
    else:
        {"plain": run_plain, "batch": run_batch, "large": run_large, "serve": run_serve,
         "sizes": run_sizes}[args.workload](args)


if __name__ == "__main__":
    main()
