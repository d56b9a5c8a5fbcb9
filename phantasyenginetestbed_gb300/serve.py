"""Serving over the C ABI (phe_server_*): continuous batching of ray-query and render requests
against device-resident scenes, admitted under a device-memory budget, with per-request latency."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as _n
from .native import LIGHT_DTYPE, RAY_HIT_DTYPE, RAY_IN_DTYPE, check, lib, ptr

REQ_CLOSEST, REQ_ANY, REQ_RENDER = 0, 1, 2


def pinned(shape, dtype):
    """A numpy array in page-locked host memory (asynchronous copies need it)."""
    import torch
    nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
    t = torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True)
    arr = t.numpy()[:nbytes].view(dtype).reshape(shape)
    _PINNED[arr.ctypes.data] = t   # the view does not own the pinned buffer: keep it alive
    return arr


_PINNED: dict = {}


class Server:
    def __init__(self, memory_budget=120 << 30, max_in_flight=256, render_slots=4, max_render_pixels=1920 * 1080,
                 max_lights=4, serial=False, batch_window_us=0):
        cfg = _n.ServerConfig()
        lib().phe_server_default_config(C.byref(cfg))
        cfg.memoryBudget = memory_budget
        cfg.maxInFlight = max_in_flight
        cfg.renderSlots = render_slots
        cfg.maxRenderPixels = max_render_pixels
        cfg.maxLights = max_lights
        cfg.serial = 1 if serial else 0
        cfg.batchWindowUs = batch_window_us
        h = C.c_void_p()
        check(lib().phe_server_create(C.byref(cfg), C.byref(h)), "phe_server_create")
        self.handle = h
        self._keep = {}
        self._scenes = []

    def add_scene(self, scene) -> int:
        i = C.c_uint32()
        check(lib().phe_server_add_scene(self.handle, scene.handle, C.byref(i)), "phe_server_add_scene")
        self._scenes.append(scene)
        return int(i.value)

    def _submit(self, req, keep) -> int:
        rid = C.c_uint64()
        check(lib().phe_server_submit(self.handle, C.byref(req), C.byref(rid)), "phe_server_submit")
        self._keep[int(rid.value)] = keep
        return int(rid.value)

    def submit_rays(self, scene_id: int, rays: np.ndarray, out: np.ndarray, kind: int = REQ_CLOSEST) -> int:
        assert rays.dtype == RAY_IN_DTYPE
        assert out.nbytes >= len(rays) * (1 if kind == REQ_ANY else RAY_HIT_DTYPE.itemsize)
        req = _n.Request()
        req.kind, req.scene, req.numRays = kind, scene_id, len(rays)
        req.rays, req.out = ptr(rays), ptr(out)
        return self._submit(req, (rays, out))

    def submit_render(self, scene_id: int, res, spp: int, cam: _n.CameraDef, cam_pos, lights: np.ndarray,
                      seed: int, out: np.ndarray) -> int:
        lights = np.ascontiguousarray(lights, LIGHT_DTYPE)
        assert out.nbytes >= res[0] * res[1] * 16
        req = _n.Request()
        req.kind, req.scene, req.spp = REQ_RENDER, scene_id, spp
        req.resX, req.resY = int(res[0]), int(res[1])
        req.out = ptr(out)
        req.cam = cam
        req.camPos[:] = [float(x) for x in cam_pos]
        req.numLights = len(lights)
        req.lights = ptr(lights)
        req.seed = seed
        return self._submit(req, (out, lights))

    def poll(self, rid: int):
        st = _n.RequestStats()
        s = lib().phe_server_poll(self.handle, rid, C.byref(st))
        if s == _n.PHE_ERR_NOT_READY:
            return None
        check(s, "phe_server_poll")
        return st

    def wait(self, rid: int):
        st = _n.RequestStats()
        check(lib().phe_server_wait(self.handle, rid, C.byref(st)), "phe_server_wait")
        return st

    def drain(self) -> None:
        check(lib().phe_server_drain(self.handle), "phe_server_drain")

    def release(self, rid: int) -> None:
        check(lib().phe_server_release(self.handle, rid), "phe_server_release")
        self._keep.pop(rid, None)

    def cancel(self, rid: int) -> bool:
        """Cancels a request not yet admitted (True); False when it is already admitted or done."""
        s = lib().phe_server_cancel(self.handle, rid)
        if s == _n.PHE_ERR_NOT_READY:
            return False
        check(s, "phe_server_cancel")
        return True

    def stats(self):
        st = _n.ServerStats()
        check(lib().phe_server_get_stats(self.handle, C.byref(st)), "phe_server_get_stats")
        return {"waves": st.waves, "rays_completed": st.raysCompleted, "bytes_in_use": st.bytesInUse,
                "pending": st.pending, "in_flight": st.inFlight}

    def close(self) -> None:
        if getattr(self, "handle", None):
            check(lib().phe_server_destroy(self.handle), "phe_server_destroy")
            self.handle = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
