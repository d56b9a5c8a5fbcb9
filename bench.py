"""Benchmark of the ray-cast hot path on GB300: the wavefront frame of the 155K-triangle scene.

One step = one frame at 1920x1080: primary closest hit -> shading + one any-hit shadow ray per
light -> one cosine-weighted bounce per hit (closest hit) -> shading + shadow rays -> resolve ->
TAA, replayed from a CUDA graph. The metric is rays cast per second over all passes (Mrays/s);
per-pass rates and per-frame p50/p99 latency are reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The scene's SBVH comes from the reference's own host builder (buildStaticFrom + sanitizeBVH,
StaticBVHBuilder.cpp:213-260, compiled from the reference sources staged in baseline/_ref): the tree a
drop-in caller of the reference's ray-cast path hands the library. Building it is input preparation,
outside every timed region, like generating the scene; where the reference sources are absent the
project's own SBVH builder stands in, and `config.bvh_builder` says which.

--impl reference times the reference's CPU ray-cast path on the host cores: the reference's own
castRay (BVHTraversal.hpp:37-128, compiled from its sources) over exactly the rays each frame casts
(primary and bounce rays closest hit, shadow rays any hit as castRay != miss), with all host threads;
the rays themselves are produced untimed by the oracle's frame. Where the reference sources are
absent it falls back to the oracle's restatement of castRay (pinned bit for bit, tests/test_oracle.py)
and says so (`cpu_baseline.kind` "port").
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
LAYOUTS = {"binary": 0, "wide4": 1, "wide8": 2}
DEFAULT_LAYOUT = "binary"
REF_BUDGET_S = 60.0   # host seconds the reference arm spends in its timed steps
CPU_LEG_BUDGET_S = 12.0   # host seconds of the cpu_baseline leg of the GPU arm
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
    ap.add_argument("--frame-parts", type=int, default=2, choices=(1, 2, 3, 4),
                    help="frame: the tile rows dealt to this many overlapping parts (same bytes); 1 = whole")
    ap.add_argument("--frames-in-flight", type=int, default=1, choices=(1, 2),
                    help="frame: 2 = consecutive frames overlap on the renderer's own streams (same bytes); "
                         "with 1, the line also reports 2 in flight without L2 flushes as a secondary figure")
    ap.add_argument("--sort-window", type=int, default=0, help="bin bounce rays by octant in windows of N (0 = off)")
    ap.add_argument("--shadows", choices=["merged", "beside", "in-order"], default="merged",
                    help="shadow-pass schedule: one pass over both queues after the bounce pass (default), the "
                         "primary shadow pass beside the bounce pass, or each after its own pass")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="frame: skip the compact batched and served runs after the frame's measurement")
    ap.add_argument("--layout", choices=["binary", "wide4", "wide8"], default=DEFAULT_LAYOUT,
                    help="node layout of the frame's scene (every layout gives the same results)")
    ap.add_argument("--workload", choices=["frame", "plain", "batch", "large", "serve", "sizes"], default="frame",
                    help="frame (default, the headline): 1080p wavefront frame; batch: 64 uneven batches over 4 "
                         "scenes in one launch vs 64 plain launches; large: 8.6M-triangle scene, 4096x4096, 4 "
                         "lights (16M diffuse + 16M shadow rays per launch); serve: Poisson request arrivals through the serving loop; sizes: launch time "
                         "against rays per launch (16K..16M) for each ray-cast entry point")
    ap.add_argument("--res", type=int, default=4096, help="large: width and height of the primary pass")
    ap.add_argument("--rays", type=int, default=16 << 20, help="large: rays per diffuse / shadow launch")
    ap.add_argument("--rates", default="200,500,1000,2000,4000,8000",
                    help="serve: arrival rates (requests/s); 2000 and above saturate the serial baseline")
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


class ReferenceTree:
    """An SBVH in the reference layout with its slot -> input-triangle map."""

    def __init__(self, nodes, verts, slot_to_tri):
        self.nodes, self.verts, self.slot_to_tri = nodes, verts, slot_to_tri

    def slot_datas(self, datas):
        return np.ascontiguousarray(datas[self.slot_to_tri])


def reference_tree(s):
    """The scene's SBVH from the reference's own host builder, or None where the reference sources were
    not present when the harness was built. Input preparation (untimed); the GPU arm's timed path runs
    only libphe_gb300.so."""
    from oracle import oracle as O
    if not O.ref_available():
        return None
    nodes, verts, s2t = O.ref_build_sbvh(s.tri_verts)
    return ReferenceTree(nodes, verts, s2t)


BUILDER_REFERENCE = "reference buildStaticFrom + sanitizeBVH (StaticBVHBuilder.cpp:213-260), compiled from its sources"
BUILDER_PROJECT = "this project's SBVH builder (the reference sources were not present)"


def frame_inputs():
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300.renderer import make_lights
    s = P.standard_scene(SCENE)
    t = time.perf_counter()
    b = reference_tree(s)
    builder = BUILDER_REFERENCE
    if b is None:
        b, builder = P.build_sbvh(s.tri_verts), BUILDER_PROJECT
    build_s = time.perf_counter() - t
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
    return s, b, cam_pos, lights, build_s, builder


def cpu_castray_rate(s, b, cam_pos, lights, budget_s, steps, first_frame=0):
    """The CPU ray-cast path on all host threads over the frame's own rays. Each step takes frame
    first_frame + k, has the oracle's frame produce (untimed) the rays of a band of rows of it — primary,
    primary shadow, bounce and bounce shadow rays — and times casting exactly those rays: the
    reference's castRay compiled from its sources (closest hit for primary and bounce rays; castRay !=
    miss for the shadow rays), or the oracle's restatement where the reference is absent. The band
    (moving down the frame) is sized so that the timed steps take about budget_s.
    Returns (Mrays/s, kind, threads, rows per band, per-step seconds)."""
    from oracle import oracle as O
    import phantasyenginetestbed_gb300 as P
    cam = O.camera_def(cam_pos, CAM_DIR, CAM_UP, math.radians(60.0), RES)
    datas = b.slot_datas(s.datas)
    threads = O.threads()
    kind = "reference" if O.ref_available() else "port"

    def band_rays(f, rows):
        dump = [np.empty(RES[0] * (rows[1] - rows[0]), O.RAY_IN_DTYPE) for _ in range(4)]
        O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, RES, P.halton_jitter(f), cam_pos, SEED, f,
                       nthreads=threads, rows=rows, dump=dump)
        return dump

    def cast(dump):
        closest = np.concatenate([dump[0], dump[2]])
        shadow = np.concatenate([dump[1], dump[3]])
        t = time.perf_counter()
        if kind == "reference":
            O.ref_cast_rays(b.nodes, b.verts, closest, nthreads=threads)
            O.ref_any_rays(b.nodes, b.verts, shadow, nthreads=threads)
        else:
            O.cast_rays(b.nodes, b.verts, closest, nthreads=threads)
            O.any_rays(b.nodes, b.verts, shadow, nthreads=threads)
        return time.perf_counter() - t, len(closest) + len(shadow)

    # Calibration on a 64-row band (untimed): rays per row and the rate.
    el, n = cast(band_rays(first_frame, (RES[1] // 2 - 32, RES[1] // 2 + 32)))
    rate = n / max(el, 1e-6)
    rows = int(max(8, min(RES[1], budget_s / steps * rate / (n / 64))))
    rays, times = 0, []
    for k in range(steps):
        r0 = (k * rows) % RES[1]
        el, n = cast(band_rays(first_frame + k, (r0, min(RES[1], r0 + rows))))
        times.append(el)
        rays += n
    return rays / sum(times) / 1e6, kind, threads, rows, times


FRAME_WORKLOAD = (f"wavefront frame {RES[0]}x{RES[1]}: primary closest -> shade + 1 any-hit shadow ray per light -> "
                  "cosine bounce closest -> shade + shadow -> resolve + TAA")
FRAME_DATA = "synthetic (seeded heightfield + cubes scene, 155,072 triangles; the reference's Sponza is not in its tree)"


L2_NOTE = "GPU arm: L2 flushed (512 MiB write) before every timed frame"


def frame_config(s, b, builder, world) -> dict:
    """The frame workload's identifying keys, identical in both arms (the GPU arm's node layout is
    reported beside them, under "frame")."""
    return {"workload": FRAME_WORKLOAD, "scene": SCENE, "triangles": int(len(s.tri_verts)),
            "resolution": f"{RES[0]}x{RES[1]}", "bvh_builder": builder, "bvh_nodes": int(len(b.nodes)),
            "bvh_slots": int(len(b.verts)), "lights": 1, "seed": SEED, "l2": L2_NOTE, "parallelism": f"replicas x{world}"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    s, b, cam_pos, lights, build_s, builder = frame_inputs()
    value, kind, threads, rows, times = cpu_castray_rate(s, b, cam_pos, lights, REF_BUDGET_S, args.steps,
                                                         first_frame=args.warmup)
    total = sum(times)
    lat = sorted(t * 1e3 for t in times)
    what = ("the reference's castRay compiled from its sources (BVHTraversal.hpp:37-128)" if kind == "reference"
            else "the oracle's restatement of castRay (the reference sources were not present)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": FRAME_DATA,
        "config": frame_config(s, b, builder, world),
        "sbvh_build_s": round(build_s, 2),
        "latency_ms": {"p50": round(lat[len(lat) // 2], 3), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3)},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": kind,
                         "sample": (f"{args.steps} frames of the {RES[0]}x{RES[1]} workload: per frame the rays of a "
                                    f"band of {rows} rows (moving down the frame; primary, shadow, bounce and bounce-"
                                    f"shadow rays as the frame casts them, produced untimed by the oracle's frame) "
                                    f"cast through {what}; shading is not timed")},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# frame pass -> its kernel function and the committed ncu summary of that kernel on this workload
PASS_KERNEL = {"primary": "primary_kernel", "bounce": "bounce_kernel", "shadows": "any_queue_kernel",
               "primary_shadow": "any_queue_kernel", "bounce_shadow": "any_queue_kernel",
               "primary_trace": "primary_trace_kernel", "bounce_trace": "bounce_trace_kernel"}


def frame_roofline(dominant, entry, clock, num_sms, builder, layout) -> dict:
    """Roofline of the dominant frame kernel. The frame's scene is L2-resident, so no memory roofline
    binds; the limit is instruction issue (4 warp instructions per SM cycle). achieved = the kernel's
    warp instructions per launch (the ncu count of that kernel on this workload, per ray, times the rays
    of the live launch) / (the live CUDA-event launch duration x SMs x the median SM clock sampled under
    load). Beside it: SIMD efficiency, DRAM / L2 / L1 fractions and DRAM bytes per launch from the same
    ncu capture, and the HBM-effective figure (algorithmic bytes / live duration / measured HBM copy
    peak), which counts bytes mostly served by L1 and L2."""
    kernel = PASS_KERNEL.get(dominant, dominant)
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peaks = json.loads(peaks_path.read_text()) if peaks_path.exists() else {}
    hbm_peak, peak_src = (float(peaks["hbm_gbs"]), "measured") if "hbm_gbs" in peaks else (6800.0, "fallback")
    mhz = clock.get("sm_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
    out = {"bound": "issue", "kernel": kernel, "pass": dominant, "achieved": None, "peak": 4.0,
           "unit": "warp instructions / SM cycle", "frac": None, "traffic": None,
           "hbm_effective": {"achieved": entry.get("GB_s"), "peak": hbm_peak, "unit": "GB/s", "peak_source": peak_src,
                             "frac": round(entry["GB_s"] / hbm_peak, 4) if entry.get("GB_s") else None}}
    prof = ROOT / "profiles" / "ncu_kernels.json"
    nc = json.loads(prof.read_text()).get(f"{kernel}/{layout}") if prof.exists() else None
    if nc and nc.get("bvh_builder") == builder:
        inst = nc["warp_inst_per_ray"] * entry["rays"]
        ipc = inst / (entry["ms"] * 1e-3 * num_sms * mhz * 1e6)
        out.update({"achieved": round(ipc, 3), "frac": round(ipc / 4.0, 4), "traffic": nc.get("dram_bytes_per_launch"),
                    "traffic_rays": nc.get("rays_per_launch"), "simd_efficiency": nc.get("simd_efficiency"),
                    "dram_frac": nc.get("dram_frac"), "l2_frac": nc.get("l2_frac"), "l1_frac": nc.get("l1_frac"),
                    "ncu_inst_per_active_cycle": nc.get("inst_per_active_cycle"), "source": nc.get("source"),
                    "how": f"{nc['warp_inst_per_ray']:.1f} warp instructions per ray (ncu) x {entry['rays']:.0f} rays / "
                           f"({entry['ms']:.4f} ms x {num_sms} SMs x {mhz:.0f} MHz)"})
    else:
        out["note"] = f"no ncu summary of {kernel} on this tree and layout ({layout}) in profiles/ncu_kernels.json"
    return out


def frame_issue(stage_rays, ms_per_frame, clock, num_sms, builder, layout) -> dict | None:
    """Issue use of the whole frame: the warp instructions of its three traversal kernels (ncu counts per
    ray on this workload times the frame's rays of each pass; the resolve, ~1% of them, left out) / (the
    frame time x SMs x the median SM clock). It counts what the overlap of a split frame's parts adds,
    which the per-kernel roofline of whole-frame kernels does not see."""
    prof = ROOT / "profiles" / "ncu_kernels.json"
    if not prof.exists():
        return None
    nc = json.loads(prof.read_text())
    rays = {"primary_kernel": stage_rays["primary"], "bounce_kernel": stage_rays["bounce"],
            "any_queue_kernel": stage_rays["primary_shadow"] + stage_rays["bounce_shadow"]}
    inst = 0.0
    for kernel, n in rays.items():
        e = nc.get(f"{kernel}/{layout}")
        if not e or e.get("bvh_builder") != builder:
            return None
        inst += e["warp_inst_per_ray"] * n
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peaks = json.loads(peaks_path.read_text()) if peaks_path.exists() else {}
    mhz = clock.get("sm_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
    ipc = inst / (ms_per_frame * 1e-3 * num_sms * mhz * 1e6)
    return {"achieved": round(ipc, 3), "peak": 4.0, "unit": "warp instructions / SM cycle", "frac": round(ipc / 4.0, 4),
            "warp_inst_per_frame": round(inst), "how": f"{inst / 1e6:.1f} M warp instructions per frame (ncu counts x this "
            f"frame's rays) / ({ms_per_frame:.4f} ms x {num_sms} SMs x {mhz:.0f} MHz)"}


def two_in_flight(r, frame, stream, first, steps, rays_per_frame, parts=1):
    """Secondary figures with two frames in flight (consecutive frames overlapping on the renderer's own
    streams, the same bytes as one at a time): device throughput over `steps` frames (CUDA events from
    before the first frame to the join after the last), per-frame GPU latency from the renderer's
    records, and end to end with the colour image read back asynchronously every frame. No L2 flush
    between frames: the frames overlap, so there is no point between them, and a flush on the caller's
    stream would run inside the next frame."""
    import torch
    from phantasyenginetestbed_gb300.renderer import READ_COLOR
    r.set_frame_parts(1)   # the two modes do not combine
    r.set_frames_in_flight(2)
    try:
        for k in range(100):   # the first pipelined frames after the switch run slower in some runs
            frame(first + k)
        torch.cuda.synchronize()
        # the latency pass first: in some runs of this process the first pass after the switch ran ~15%
        # slower (never in a standalone process), so the device-timed pass comes second
        r.set_seed(SEED, first)
        r.set_latency_recording(True)
        for k in range(steps):
            frame(first + k)
        lat = sorted(float(x) for x in r.frame_latencies())
        r.set_latency_recording(False)
        region = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        torch.cuda.synchronize()
        r.set_seed(SEED, first)
        region[0].record(stream)
        for k in range(steps):
            frame(first + k)
        r.join(stream)
        region[1].record(stream)
        torch.cuda.synchronize()
        ms = region[0].elapsed_time(region[1])
        host_imgs = [torch.empty((RES[1], RES[0], 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
        torch.cuda.synchronize()
        r.set_seed(SEED, first)
        t0 = time.perf_counter()
        for k in range(steps):
            frame(first + k)
            r.read_async(host_imgs[k & 1], READ_COLOR, stream=stream)
        r.read_wait()
        e2e_s = time.perf_counter() - t0
    finally:
        r.set_frames_in_flight(1)
        r.set_frame_parts(parts)
    return {"Mrays_s": round(rays_per_frame * steps / (ms / 1e3) / 1e6, 2), "ms_per_frame": round(ms / steps, 4),
            "latency_ms": {"p50": round(lat[len(lat) // 2], 4), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 4),
                           "of": "per frame on the GPU, first kernel start to resolve end"},
            "e2e_Mrays_s": round(rays_per_frame * steps / e2e_s / 1e6, 2),
            "l2": "not flushed between frames: overlapping frames have no point between them"}


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
    s, b, cam_pos, lights, build_s, builder = frame_inputs()
    scene = P.Scene(b.nodes, b.verts, b.slot_datas(s.datas), s.materials)
    scene.set_layout(LAYOUTS[args.layout])
    r = CudaTracerRenderer(use_graph=not args.no_graph)
    r.set_pipeline(fused=args.pipeline == "fused", refill=args.refill, sort_window=args.sort_window)
    r.set_shadow_schedule({"in-order": 0, "beside": 1, "merged": 2}[args.shadows])
    r.setStaticScene(scene)
    r.setTargetResolution(RES)
    r.set_frame_parts(args.frame_parts)
    r.set_frames_in_flight(args.frames_in_flight)
    r.set_seed(SEED, 0)
    r.resetTAA()
    stream = torch.cuda.current_stream()
    inflight = args.frames_in_flight
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")   # 4x the 126 MiB L2

    def frame(f):
        r.updateCamera(cam_pos, CAM_DIR, CAM_UP, 60.0, P.halton_jitter(f))
        r.render(lights, stream=stream)

    for f in range(args.warmup):
        frame(f)
    torch.cuda.synchronize()
    first = args.warmup

    # Timed region: K frames, L2 flushed before each. One frame in flight: CUDA events around each
    # frame on the render stream (the flushes fall outside them). Two in flight: frames overlap on the
    # renderer's streams, so the region runs from before the first flush to the join after the last
    # frame (flushes included); per-frame latency comes from the renderer's latency records of a
    # second, identical pass.
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    region = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    r.set_seed(SEED, first)
    with ClockSampler(local) as clocks:
        if inflight == 1:
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                frame(first + k)
                ends[k].record(stream)
        else:
            region[0].record(stream)
            for k in range(args.steps):
                flush.zero_()
                frame(first + k)
            r.join(stream)
            region[1].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    if inflight == 1:
        per = [a.elapsed_time(e) for a, e in zip(starts, ends)]
        total_ms = sum(per)
    else:
        total_ms = region[0].elapsed_time(region[1])
        r.set_seed(SEED, first)
        r.set_latency_recording(True)
        for k in range(args.steps):
            flush.zero_()
            frame(first + k)
        per = [float(x) for x in r.frame_latencies()]
        r.set_latency_recording(False)
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
    overlap = (two_in_flight(r, frame, stream, first, args.steps, rays_per_frame, args.frame_parts)
               if inflight == 1 else None)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    work = json.loads((ROOT / "profiles" / "work_per_ray.json").read_text())["trees"][
        "reference" if builder == BUILDER_REFERENCE else "project"]["stages"]
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
    lat = sorted(per)
    clock = clocks.summary()
    num_sms = torch.cuda.get_device_properties(local).multi_processor_count
    roofline = frame_roofline(dominant, per_kernel[dominant], clock, num_sms, builder, args.layout)
    roofline["frame_issue"] = frame_issue(stage_rays, total_ms / args.steps, clock, num_sms, builder, args.layout)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, kind, cores, rows, times = cpu_castray_rate(s, b, cam_pos, lights, CPU_LEG_BUDGET_S, 4, first_frame=first)
        what = "the reference's castRay compiled from its sources" if kind == "reference" else "the castRay restatement"
        cpu = {"value": round(v, 3), "unit": "Mrays/s", "cores": cores, "kind": kind,
               "sample": (f"4 frames x a band of {rows} rows: the band's primary, shadow, bounce and bounce-shadow rays "
                          f"(produced untimed by the oracle's frame) cast through {what} ({sum(times):.1f} s)")}
    launches_per_frame = len(names) * args.frame_parts   # each part launches the frame's kernels
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": FRAME_DATA,
        "config": frame_config(s, b, builder, world),
        "frame": {"rays_per_frame": round(rays_per_frame, 1), "rays_by_pass": {k: round(v, 1) for k, v in stage_rays.items()},
                  "frame_parts": args.frame_parts, "frames_in_flight": inflight, "two_frames_in_flight": overlap,
                  "cuda_graph": not args.no_graph and inflight == 1,
                  "pipeline": args.pipeline, "refill_threshold": args.refill,
                  "sort_window": args.sort_window, "sbvh_build_s": round(build_s, 2), "node_layout": args.layout,
                  "shadow_schedule": args.shadows if args.pipeline == "fused" else "in-order"},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 4), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 4),
                       "of": ("per frame, CUDA events around it" if inflight == 1 else
                              "per frame on the GPU, first kernel start to resolve end, 2 frames in flight")},
        "passes": per_kernel,
        "roofline": roofline,
        "clocks": clock,
        "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s",
                "h2d_bytes_per_step": int(native.lib().phe_renderer_frame_param_bytes()) * args.frame_parts,
                "d2h_bytes_per_step": RES[0] * RES[1] * 16,
                "mode": "pipelined: colour image read back asynchronously (two pinned host images) while the "
                        "next frames render; clock stops when the last image is in host memory",
                "blocking_value": round(e2e_blocking, 2)},
        "gpu_launches": launches_per_frame * args.steps,
        "cpu_baseline": cpu,
    }
    if world == 1 and not args.no_secondary:
        line["secondary"] = secondary_measures()
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------------------------
# Additional workloads (not the headline line): uneven batches, large incoherent scene, serving.
# ---------------------------------------------------------------------------------------------

SECONDARY_SERVE_RATE = 4000.0   # requests/s: saturates the serial server, not the continuous one


def secondary_measures() -> dict:
    """Compact runs of the other workloads, after the frame's timed region, so that the frame line also
    carries them: the uneven batch mix (measure_batch: autotuned graph launch vs 64 plain launches, 10
    timed steps each, L2 flushed), the large incoherent workload on the binary layout (measure_large: 10
    timed launches per pass, L2 flushed) and Poisson serving at one rate that saturates the serial server
    (measure_serve: 2 s of arrivals, continuous batching vs serial). A failure is reported in place of
    that entry and leaves the frame line intact."""
    out = {}
    try:
        b = measure_batch(10, 3)
        out["batch"] = {"workload": "64 ray batches of 1K-1M rays over 4 scenes (10K-2M triangles), 70/30 closest/any",
                        "rays": b["rays"], "batched_graph": {k: b["batched_graph"][k] for k in ("ms", "Mrays_s", "params")},
                        "plain_64_launches": {k: b["plain_64_launches"][k] for k in ("ms", "Mrays_s")},
                        "speedup_vs_plain": b["speedup_vs_plain"], "speedup_vs_synchronised": b["speedup_vs_synchronised"],
                        "l2": b["l2"]}
    except Exception as e:   # noqa: BLE001 - reported in the line
        out["batch"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    try:
        lg = measure_large(4096, 16 << 20, 10, 3, layout_names=("binary",))
        out["large"] = {"workload": f"{lg['triangles']:,} triangles: 16M diffuse closest-hit rays from the hits of a "
                                    "4096x4096 primary pass, then 16M any-hit shadow rays over 4 lights, one launch each",
                        "primary": {k: lg["primary"][k] for k in ("ms", "Mrays_s")},
                        "diffuse_closest": {k: lg["layouts"]["binary"]["diffuse_closest"][k] for k in ("ms", "Mrays_s")},
                        "shadow_any": {k: lg["layouts"]["binary"]["shadow_any"][k] for k in ("ms", "Mrays_s")},
                        "hbm_frac": {p: r["frac"] for p, r in lg.get("roofline", {}).items()},
                        "l2": lg["l2"]}
    except Exception as e:   # noqa: BLE001 - reported in the line
        out["large"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    try:
        sv = measure_serve([SECONDARY_SERVE_RATE], 2.0, 8, 0, burst_too=False)
        row = sv["rates"][str(int(SECONDARY_SERVE_RATE))]
        out["serve"] = {"workload": "Poisson arrivals of render and ray-query requests over 8 scenes "
                                    f"({min(sv['scenes_triangles']):,}-{max(sv['scenes_triangles']):,} triangles)",
                        "rate_req_s": SECONDARY_SERVE_RATE, "arrivals_s": 2.0,
                        "continuous": row["continuous"], "serial": row["serial"],
                        "speedup": round(row["continuous"]["Mrays_s"] / max(row["serial"]["Mrays_s"], 1e-9), 3)}
    except Exception as e:   # noqa: BLE001 - reported in the line
        out["serve"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return out

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
    for layout, lname in ((0, "binary"), (1, "wide4"), (2, "wide8")):
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
    print(json.dumps(measure_batch(args.steps, args.warmup, save_tuning_to=ROOT / "profiles" / "batch_autotune.json")),
          flush=True)


def measure_batch(steps, warmup, save_tuning_to=None):
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
    if save_tuning_to is not None:
        save_tuning(save_tuning_to, best, best_ms, table,
                    command=f"python bench.py --workload batch --steps {steps} --warmup {warmup} "
                            "(phe_batch_autotune, repeats=3, cold L2)")
    batch.set_params(block_size=best["blockSize"], blocks_per_sm=best["blocksPerSM"], order=best["order"], use_graph=True,
                     layout=best["layout"], stack_shared=best["stackShared"], sort_window=best["sortWindow"])
    for _ in range(warmup):
        batch.launch(stream)
    t_batched = _timed(lambda: batch.launch(stream), steps, stream, flush)

    def plain():
        for si, kind, n, d_rays, out in items:
            (P.cast_closest if kind == CLOSEST else P.cast_any)(scenes[si], d_rays, out, n, stream=stream)

    def plain_sync():
        for si, kind, n, d_rays, out in items:
            (P.cast_closest if kind == CLOSEST else P.cast_any)(scenes[si], d_rays, out, n, stream=stream)
            torch.cuda.synchronize()

    for _ in range(warmup):
        plain()
    t_plain = _timed(plain, steps, stream, flush)
    steps_sync = max(3, steps // 5)
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
    for x in [batch] + scenes:   # the batch holds the scene handles
        x.close()
    return line


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


def large_rays(s, b, prim_rays, prim_hits, n, lights, seed):
    """The large workload's secondary rays, from the hit points of the primary pass (cycled where fewer
    than n pixels hit): n diffuse rays, cosine-weighted about the hit triangle's geometric normal
    (flipped to face the incoming ray), directions from a seeded PCG64 stream; and n any-hit shadow
    rays, ray i from hit point i // 4 toward light i % 4, tMin 1e-3, tMax = the distance to the light."""
    import phantasyenginetestbed_gb300 as P
    hit = prim_hits["triangleIndex"] != 0xFFFFFFFF
    r, h = prim_rays[hit], prim_hits[hit]
    pos = r["origin"] + r["dir"] * h["t"][:, None]
    tv = b.verts[h["triangleIndex"]]
    nrm = np.cross(tv["v1"][:, :3] - tv["v0"][:, :3], tv["v2"][:, :3] - tv["v0"][:, :3])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(((nrm * r["dir"]).sum(1) > 0)[:, None], -nrm, nrm).astype(np.float32)
    H = len(pos)
    rng = np.random.default_rng(seed)   # PCG64
    idx = np.arange(n) % H
    r1, r2 = rng.random(n, np.float32), rng.random(n, np.float32)
    phi = 2.0 * np.pi * r1
    st, ct = np.sqrt(r2), np.sqrt(1.0 - r2)
    nn = nrm[idx]
    up = np.where(np.abs(nn[:, 2:3]) < 0.999, np.array([0, 0, 1], np.float32), np.array([1, 0, 0], np.float32))
    u = np.cross(up, nn)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(nn, u)
    d = u * (st * np.cos(phi))[:, None] + v * (st * np.sin(phi))[:, None] + nn * ct[:, None]
    diffuse = np.zeros(n, P.RAY_IN_DTYPE)
    diffuse["origin"] = pos[idx]
    diffuse["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    diffuse["tMin"], diffuse["tMax"] = np.float32(1e-3), np.float32(3.4028235e38)
    lp = np.asarray([l["pos"] for l in lights], np.float32)
    o = pos[(np.arange(n) // 4) % H]
    to = lp[np.arange(n) % 4] - o
    dist = np.linalg.norm(to, axis=1)
    shadow = np.zeros(n, P.RAY_IN_DTYPE)
    shadow["origin"] = o
    shadow["dir"] = (to / dist[:, None]).astype(np.float32)
    shadow["tMin"], shadow["tMax"] = np.float32(1e-3), dist.astype(np.float32)
    return diffuse, shadow, H


def run_large(args):
    print(json.dumps(measure_large(args.res, args.rays, args.steps, args.warmup)), flush=True)


def measure_large(res_side, N, steps, warmup, layout_names=("binary", "wide4", "wide8")):
    """The large incoherent workload: 8.63M-triangle scene (2048x2048-cell heightfield + 20,000 cubes,
    world x32). A 4096x4096 pinhole primary pass gives the hit points; then ONE launch of 16M diffuse
    closest-hit rays from them (cosine-weighted, seeded PCG64 directions) and ONE launch of 16M any-hit
    shadow rays toward 4 point lights, each timed over `steps` launches from a cold L2 (the scene is
    ~0.9 GB, 7x the L2), on every node layout the scene offers. HBM traffic per launch comes from a
    one-kernel ncu capture (profiles/large_workload_ncu.md)."""
    import torch
    import phantasyenginetestbed_gb300 as P
    from phantasyenginetestbed_gb300.renderer import make_lights
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    res = (res_side, res_side)
    s, b, build_s = _scene_with_bvh("c4_2048_20000")
    scene = P.Scene(b.nodes, b.verts)
    k = s.scale
    cam = P.camera_def((0.5 * k, -0.3 * k, 0.6 * k), CAM_DIR, CAM_UP, 60.0, res)
    lights = make_lights(np.array([[0.5, 0.5, 2.0], [0.1, 0.1, 1.0], [0.9, 0.2, 1.5], [0.3, 0.9, 0.8]], np.float32)
                         * np.float32(k), range_=1000.0 * k)
    npix = res[0] * res[1]
    prim = torch.empty(npix * 32, dtype=torch.uint8, device="cuda")
    P.gen_primary_rays(prim, cam, res, order=1)
    prim_hits = torch.empty(npix * 16, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    P.cast_closest(scene, prim, prim_hits, npix, stream=stream)
    torch.cuda.synchronize()
    t_prim = statistics.median(_timed(lambda: P.cast_closest(scene, prim, prim_hits, npix, stream=stream), 3, stream, flush))
    diffuse, shadow, H = large_rays(s, b, prim.cpu().numpy().view(P.RAY_IN_DTYPE),
                                    prim_hits.cpu().numpy().view(P.RAY_HIT_DTYPE), N, lights, SEED)
    d_diffuse = torch.from_numpy(diffuse.view(np.uint8)).cuda()
    d_shadow = torch.from_numpy(shadow.view(np.uint8)).cuda()
    hits = torch.empty(N * 16, dtype=torch.uint8, device="cuda")
    vis = torch.empty(N, dtype=torch.uint8, device="cuda")
    layouts = {}
    lay0, avail = scene.layout()
    for layout, name in ((0, "binary"), (1, "wide4"), (2, "wide8")):
        if name not in layout_names or (layout and not (avail & layout)):
            continue
        scene.set_layout(layout)
        row = {}
        for pas, fn in (("diffuse_closest", lambda: P.cast_closest(scene, d_diffuse, hits, N, stream=stream)),
                        ("shadow_any", lambda: P.cast_any(scene, d_shadow, vis, N, stream=stream))):
            for _ in range(warmup):
                fn()
            t = _timed(fn, max(3, min(steps, 20)), stream, flush)
            m = statistics.median(t)
            row[pas] = {"ms": round(m, 3), "Mrays_s": round(N / m / 1e3, 1), "latency_ms": _percentiles(t)}
        layouts[name] = row
    scene.set_layout(0)
    torch.cuda.synchronize()
    line = {"workload": "large", "metric": METRIC, "unit": "Mrays/s", "triangles": int(len(s.tri_verts)),
            "bvh_builder": "this project's SBVH builder", "bvh_nodes": int(len(b.nodes)), "bvh_slots": int(len(b.verts)),
            "sbvh_build_s": round(build_s, 1), "scene_bytes": scene.device_bytes(),
            "primary": {"res": res, "rays": npix, "hits": int(H), "ms": round(t_prim, 3),
                        "Mrays_s": round(npix / t_prim / 1e3, 1)},
            "rays_per_launch": N, "lights": 4, "layouts": layouts,
            "l2": "flushed (512 MiB write) before every timed launch"}
    ncu = ROOT / "profiles" / "large_workload_ncu.json"
    if ncu.exists():
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        roof = {}
        for pas, rec in json.loads(ncu.read_text()).get("passes", {}).items():
            ms = layouts.get(rec.get("layout", "binary"), {}).get(pas, {}).get("ms")
            if ms:
                bytes_launch = rec["dram_bytes_per_ray"] * N
                roof[pas] = {"bound": "hbm", "traffic": int(bytes_launch), "achieved": round(bytes_launch / ms / 1e6, 1),
                             "peak": hbm, "unit": "GB/s", "frac": round(bytes_launch / ms / 1e6 / hbm, 4),
                             "how": f"{rec['dram_bytes_per_ray']:.1f} DRAM bytes per ray (ncu, {rec['source']}) x {N} rays / "
                                    f"live launch time"}
        line["roofline"] = roof
    scene.close()
    return line


def run_serve(args):
    print(json.dumps(measure_serve([float(x) for x in args.rates.split(",")], args.duration, args.render_slots,
                                   args.batch_window_us)), flush=True)


def measure_serve(rates, duration, render_slots, batch_window_us, burst_too=True):
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
    for rate in rates:
        reqs = make_requests(rate, duration, int(rate))
        row = {}
        for mode in ("continuous", "serial"):
            server = Server(memory_budget=120 << 30, render_slots=render_slots, serial=(mode == "serial"),
                            batch_window_us=batch_window_us)
            ids = [server.add_scene(sc) for sc in scenes]
            row[mode] = run(server, ids, reqs)
            server.close()
        results[str(int(rate))] = row
    if burst_too:
        # Saturation: the highest rate's requests all submitted at once (makespan throughput).
        burst = {}
        reqs = make_requests(max(rates), duration, 99)
        for mode in ("continuous", "serial"):
            server = Server(memory_budget=120 << 30, render_slots=render_slots, serial=(mode == "serial"),
                            batch_window_us=batch_window_us)
            ids = [server.add_scene(sc) for sc in scenes]
            burst[mode] = run(server, ids, reqs, burst=True)
            server.close()
        burst["speedup"] = round(burst["continuous"]["Mrays_s"] / max(burst["serial"]["Mrays_s"], 1e-9), 3)
        results["burst"] = burst
    for sc in scenes:
        sc.close()
    return {"workload": "serve", "metric": METRIC, "unit": "Mrays/s",
            "scenes_triangles": [int(len(s.tri_verts)) for s, _ in built], "scene_build_s": round(build_s, 1),
            "budget_bytes": 120 << 30, "arrivals_s": duration, "render_slots": render_slots,
            "batch_window_us": batch_window_us, "rates": results}


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
