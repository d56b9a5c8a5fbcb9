"""CudaTracerRenderer: the headless renderer object over the C ABI (phe_renderer_*).

Mirrors the reference's renderer entry points (phantasy_engine/rendering/BaseRenderer.hpp:56-90,
cuda_ray_tracer/CudaTracerRenderer.hpp:14-58): setStaticScene, setTargetResolution, updateCamera,
render. render() returns a RenderResult whose buffers are device pointers instead of GL textures.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native as _n
from .native import LIGHT_DTYPE, check, lib, ptr

READ_COLOR, READ_HISTORY, READ_RAW, READ_ROUGHNESS, READ_VELOCITY = 0, 1, 2, 3, 4


@dataclass
class RenderResult:
    res: tuple
    color: int
    history: int
    raw_color: int
    roughness: int
    velocity: int | None = None   # device float2 per pixel, None while the camera stands still


def _stream(stream):
    if stream is None:
        return None
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


SHADOWS_IN_ORDER, SHADOWS_BESIDE_BOUNCE, SHADOWS_MERGED = 0, 1, 2


class CudaTracerRenderer:
    def __init__(self, use_graph: bool = False):
        h = C.c_void_p()
        check(lib().phe_renderer_create(C.byref(h)), "phe_renderer_create")
        self.handle = h
        self.res = (0, 0)
        self.scene = None
        self._materials = None
        if use_graph:
            self.set_graph(True)

    def setMaterialsAndTextures(self, materials, textures=()) -> None:
        """BaseRenderer::setMaterialsAndTextures (CudaTracerRenderer.cpp:192-239). The reference calls it
        before setStaticScene; the arrays belong to the device scene here, so they are applied to the
        current scene now and to each scene given to setStaticScene later."""
        self._materials = (materials, list(textures))
        if self.scene is not None:
            self.scene.setMaterialsAndTextures(materials, textures)

    def setStaticScene(self, scene) -> None:
        if self._materials is not None:
            scene.setMaterialsAndTextures(*self._materials)
        check(lib().phe_renderer_set_static_scene(self.handle, scene.handle), "phe_renderer_set_static_scene")
        self.scene = scene

    def setTargetResolution(self, res) -> None:
        check(lib().phe_renderer_set_target_resolution(self.handle, int(res[0]), int(res[1])),
              "phe_renderer_set_target_resolution")
        self.res = (int(res[0]), int(res[1]))

    def updateCamera(self, pos, direction, up, vfov_deg: float, pixel_offset=(0.0, 0.0)) -> None:
        check(lib().phe_renderer_update_camera(self.handle, _n.fvec(pos), _n.fvec(direction), _n.fvec(up),
                                               C.c_float(vfov_deg), C.c_float(pixel_offset[0]),
                                               C.c_float(pixel_offset[1])), "phe_renderer_update_camera")

    def set_camera_def(self, cam: _n.CameraDef, cam_pos, pixel_offset=(0.0, 0.0)) -> None:
        check(lib().phe_renderer_set_camera_def(self.handle, C.byref(cam), _n.fvec(cam_pos), C.c_float(pixel_offset[0]),
                                                C.c_float(pixel_offset[1])), "phe_renderer_set_camera_def")

    def set_seed(self, seed: int, frame: int = 0) -> None:
        check(lib().phe_renderer_set_seed(self.handle, seed, frame), "phe_renderer_set_seed")

    def set_graph(self, enable: bool) -> None:
        check(lib().phe_renderer_set_graph(self.handle, 1 if enable else 0), "phe_renderer_set_graph")

    def resetTAA(self, stream=None) -> None:
        check(lib().phe_renderer_reset_taa(self.handle, _stream(stream)), "phe_renderer_reset_taa")

    def render(self, lights: np.ndarray, stream=None) -> RenderResult:
        lights = np.ascontiguousarray(lights, LIGHT_DTYPE)
        check(lib().phe_renderer_render(self.handle, ptr(lights) if len(lights) else None, len(lights), _stream(stream)),
              "phe_renderer_render")
        r = _n.RenderResult()
        check(lib().phe_renderer_result(self.handle, C.byref(r)), "phe_renderer_result")
        return RenderResult((r.resX, r.resY), r.color, r.history, r.rawColor, r.roughness, r.velocity)

    def read(self, which: int = READ_COLOR, out: np.ndarray | None = None, stream=None) -> np.ndarray:
        W, H = self.res
        if out is None:
            out = np.empty((H, W) if which == READ_ROUGHNESS else (H, W, 2) if which == READ_VELOCITY else (H, W, 4),
                           np.float32)
        check(lib().phe_renderer_read(self.handle, which, ptr(out), _stream(stream)), "phe_renderer_read")
        return out

    def read_async(self, out: np.ndarray, which: int = READ_COLOR, stream=None) -> None:
        """Queue a read-back into `out` (pinned for overlap); the image is there after read_wait()."""
        W, H = self.res
        need = W * H * (4 if which == READ_ROUGHNESS else 8 if which == READ_VELOCITY else 16)
        if out.nbytes < need or not out.flags.c_contiguous:
            raise ValueError(f"read_async: need a contiguous buffer of {need} bytes")
        check(lib().phe_renderer_read_async(self.handle, which, ptr(out), _stream(stream)), "phe_renderer_read_async")

    def read_wait(self) -> None:
        check(lib().phe_renderer_read_wait(self.handle), "phe_renderer_read_wait")

    def ray_counts(self, stream=None) -> np.ndarray:
        c = (C.c_uint64 * 4)()
        check(lib().phe_renderer_ray_counts(self.handle, c, _stream(stream)), "phe_renderer_ray_counts")
        return np.array(list(c), np.uint64)

    def set_kernel_timing(self, enable: bool) -> None:
        check(lib().phe_renderer_set_kernel_timing(self.handle, 1 if enable else 0), "phe_renderer_set_kernel_timing")

    def kernel_times(self):
        """(summed ms per frame kernel in launch order, frames timed)."""
        ms = (C.c_double * 8)()
        k, n = C.c_uint32(), C.c_uint32()
        check(lib().phe_renderer_kernel_times(self.handle, ms, C.byref(k), C.byref(n)), "phe_renderer_kernel_times")
        return np.array(list(ms)[:k.value]), int(n.value)

    def set_pipeline(self, fused: bool = True, refill: int = 28, sort_window: int = 0) -> None:
        """fused: traversal + shading in one kernel per bounce; refill: lane-refill threshold (0..32);
        sort_window: bin bounce rays by direction octant within windows of this many rays (0 = off)."""
        check(lib().phe_renderer_set_pipeline(self.handle, 1 if fused else 0, refill, sort_window),
              "phe_renderer_set_pipeline")

    def set_frames_in_flight(self, frames: int) -> None:
        """1 (default): each frame runs on the caller's stream. 2: consecutive frames overlap on the
        renderer's own streams (same results); the caller's stream is not ordered after a frame: reads
        wait for it, join() orders a stream after the last frame."""
        check(lib().phe_renderer_set_frames_in_flight(self.handle, int(frames)), "phe_renderer_set_frames_in_flight")

    def set_frame_parts(self, parts: int) -> None:
        """1 (default): a frame's kernels run as one. 2..4: the tile rows are dealt to that many parts on
        their own streams inside the frame (same bytes); the frame still ends on the caller's stream."""
        check(lib().phe_renderer_set_frame_parts(self.handle, int(parts)), "phe_renderer_set_frame_parts")

    def join(self, stream=None) -> None:
        """Orders `stream` after the last frame (a no-op with one frame in flight)."""
        check(lib().phe_renderer_join(self.handle, _stream(stream)), "phe_renderer_join")

    def set_latency_recording(self, enable: bool) -> None:
        """With two frames in flight: record each frame's GPU latency (first kernel start to resolve end)."""
        check(lib().phe_renderer_set_latency_recording(self.handle, 1 if enable else 0),
              "phe_renderer_set_latency_recording")

    def frame_latencies(self) -> np.ndarray:
        """Latencies (ms) of the frames recorded since the last call, waiting for them."""
        n = C.c_uint32(0)
        check(lib().phe_renderer_frame_latencies(self.handle, None, 0, C.byref(n)), "phe_renderer_frame_latencies")
        out = np.zeros(n.value, np.float32)
        if n.value:
            buf = out.ctypes.data_as(C.POINTER(C.c_float))
            check(lib().phe_renderer_frame_latencies(self.handle, buf, n.value, C.byref(n)), "phe_renderer_frame_latencies")
        return out[: n.value]

    def set_shadow_schedule(self, schedule: int = 2) -> None:
        """SHADOWS_IN_ORDER, SHADOWS_BESIDE_BOUNCE or SHADOWS_MERGED (default); same results."""
        check(lib().phe_renderer_set_shadow_schedule(self.handle, int(schedule)), "phe_renderer_set_shadow_schedule")

    def close(self) -> None:
        if getattr(self, "handle", None):
            check(lib().phe_renderer_destroy(self.handle), "phe_renderer_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_lights(positions, strength=(20.0, 20.0, 20.0), range_=1000.0, radius=0.0) -> np.ndarray:
    """Point lights (radius 0) with static shadows, as SphereLight (level/SphereLight.hpp:13-26)."""
    pos = np.asarray(positions, np.float32).reshape(-1, 3)
    L = np.zeros(len(pos), LIGHT_DTYPE)
    L["pos"] = pos
    L["radius"] = radius
    L["range"] = range_
    L["strength"] = strength
    L["staticShadows"] = 1
    return L


def taa_resolve(res, cur, hist, out_color, out_hist, velocity=None, prev_velocity=None, roughness=None, stream=None):
    """TAA resolve on device buffers (phe_taa_resolve)."""
    check(lib().phe_taa_resolve(int(res[0]), int(res[1]), ptr(cur), ptr(hist), ptr(velocity), ptr(prev_velocity),
                                ptr(roughness), ptr(out_color), ptr(out_hist), _stream(stream)), "phe_taa_resolve")


def postprocess(res, linear, display=None, rgba8=None, gamma=2.2, stream=None):
    """Uncharted 2 tonemap + gamma on device buffers (phe_postprocess)."""
    check(lib().phe_postprocess(int(res[0]), int(res[1]), ptr(linear), C.c_float(gamma), ptr(display), ptr(rgba8),
                                _stream(stream)), "phe_postprocess")


def scale(src_res, src, dst_res, dst=None, rgba8=None, viewport=None, stream=None):
    """Display scaling pass (scaling.frag) on device buffers (phe_scale): the `viewport` part of the
    float4 `src` image resampled to `dst_res`."""
    vw, vh = viewport or src_res
    check(lib().phe_scale(int(src_res[0]), int(src_res[1]), ptr(src), int(vw), int(vh), int(dst_res[0]),
                          int(dst_res[1]), ptr(dst), ptr(rgba8), _stream(stream)), "phe_scale")


def write_ppm(path, rgba8: np.ndarray) -> None:
    """Writes an (H, W, 4) uint8 image as binary PPM, top row first (the renderer's row 0 is the bottom)."""
    h, w = rgba8.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgba8[::-1, :, :3]).tobytes())
