"""ctypes binding of libphe_gb300.so (the C ABI declared in include/phe_gb300.h).

The library is the product: there is no Python or CPU fallback for any GPU entry point. Loading fails
loudly when the library has not been built (``python -m phantasyenginetestbed_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

# PHE_GB300_CHECKED=1 selects the checked build (device-side index checks, libphe_gb300_checked.so,
# built with `python -m phantasyenginetestbed_gb300.build --checked`).
CHECKED = os.environ.get("PHE_GB300_CHECKED") == "1"
LIB_PATH = Path(__file__).resolve().parent / ("libphe_gb300_checked.so" if CHECKED else "libphe_gb300.so")

# Status codes (include/phe_gb300.h).
PHE_OK = 0
PHE_ERR_INVALID_ARGUMENT = 1
PHE_ERR_INVALID_SCENE = 2
PHE_ERR_CUDA = 3
PHE_ERR_OUT_OF_MEMORY = 4
PHE_ERR_BUDGET = 5
PHE_ERR_TIMEOUT = 6
PHE_ERR_NOT_FOUND = 7
PHE_ERR_TOO_LARGE = 8
PHE_ERR_NOT_READY = 9
PHE_ERR_CANCELLED = 11
PHE_ERR_NO_DEVICE = 10

PTR_HOST = 0
PTR_DEVICE = 1
LAYOUT_BINARY = 0
LAYOUT_WIDE4 = 1
LAYOUT_WIDE8 = 2

# numpy views of the reference layouts
NODE_DTYPE = np.dtype([("fData", "<f4", (12,)), ("iData", "<i4", (4,))])            # phe::BVHNode, 64 B
TRI_VERTS_DTYPE = np.dtype([("v0", "<f4", (4,)), ("v1", "<f4", (4,)), ("v2", "<f4", (4,))])  # 48 B
TRI_DATA_DTYPE = np.dtype([("n0", "<f4", (3,)), ("n1", "<f4", (3,)), ("n2", "<f4", (3,)),
                           ("uv0", "<f4", (2,)), ("uv1", "<f4", (2,)), ("uv2", "<f4", (2,)),
                           ("materialIndex", "<u4")])                                 # 64 B
RAY_IN_DTYPE = np.dtype([("origin", "<f4", (3,)), ("tMin", "<f4"), ("dir", "<f4", (3,)), ("tMax", "<f4")])  # 32 B
RAY_HIT_DTYPE = np.dtype([("triangleIndex", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])  # 16 B
MATERIAL_DTYPE = np.dtype([("texIndex", "<i4", (4,)), ("albedo", "<f4", (4,)), ("roughness", "<f4"), ("metallic", "<f4"),
                           ("pad", "<f4", (2,))])
LIGHT_DTYPE = np.dtype([("pos", "<f4", (3,)), ("radius", "<f4"), ("range", "<f4"), ("strength", "<f4", (3,)),
                        ("staticShadows", "<i4")])
assert NODE_DTYPE.itemsize == 64 and TRI_VERTS_DTYPE.itemsize == 48 and TRI_DATA_DTYPE.itemsize == 64
assert RAY_IN_DTYPE.itemsize == 32 and RAY_HIT_DTYPE.itemsize == 16 and MATERIAL_DTYPE.itemsize == 48
assert LIGHT_DTYPE.itemsize == 36


class CameraDef(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("dir", C.c_float * 3), ("dX", C.c_float * 3), ("dY", C.c_float * 3)]


class Texture(C.Structure):
    """phe_texture: a RawImage-like host image (8-bit channels)."""
    _fields_ = [("data", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("bytesPerPixel", C.c_uint32),
                ("pitch", C.c_uint32)]


class SceneRecipe(C.Structure):
    _fields_ = [("gridCells", C.c_uint32), ("numCubes", C.c_uint32), ("rotatedCubes", C.c_int32),
                ("pad", C.c_uint32), ("seed", C.c_uint64)]


class SbvhParams(C.Structure):
    _fields_ = [("splitAlpha", C.c_float), ("maxDepth", C.c_int32), ("maxSpatialDepth", C.c_int32),
                ("numThreads", C.c_int32)]


class RenderResult(C.Structure):
    _fields_ = [("resX", C.c_uint32), ("resY", C.c_uint32), ("color", C.c_void_p), ("history", C.c_void_p),
                ("rawColor", C.c_void_p), ("roughness", C.c_void_p), ("velocity", C.c_void_p)]


class BatchItem(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("kind", C.c_uint32), ("count", C.c_uint32), ("pad", C.c_uint32),
                ("rays", C.c_void_p), ("out", C.c_void_p)]


class BatchParams(C.Structure):
    _fields_ = [("blockSize", C.c_int32), ("blocksPerSM", C.c_int32), ("order", C.c_int32), ("useGraph", C.c_int32),
                ("layout", C.c_int32), ("stackShared", C.c_int32), ("sortWindow", C.c_int32), ("pad", C.c_int32)]


class BatchTuningRow(C.Structure):
    _fields_ = [("params", BatchParams), ("ms", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("memoryBudget", C.c_uint64), ("maxInFlight", C.c_uint32), ("renderSlots", C.c_uint32),
                ("maxRenderPixels", C.c_uint32), ("maxLights", C.c_uint32), ("serial", C.c_int32),
                ("batchWindowUs", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("scene", C.c_uint32), ("numRays", C.c_uint32), ("spp", C.c_uint32),
                ("rays", C.c_void_p), ("out", C.c_void_p), ("resX", C.c_uint32), ("resY", C.c_uint32),
                ("numLights", C.c_uint32), ("pad", C.c_uint32), ("cam", CameraDef), ("camPos", C.c_float * 3),
                ("pad2", C.c_float), ("lights", C.c_void_p), ("seed", C.c_uint64)]


class RequestStats(C.Structure):
    _fields_ = [("submitMs", C.c_double), ("admitMs", C.c_double), ("doneMs", C.c_double), ("rays", C.c_uint64),
                ("status", C.c_int), ("pad", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("waves", C.c_uint64), ("raysCompleted", C.c_uint64), ("bytesInUse", C.c_uint64),
                ("pending", C.c_uint32), ("inFlight", C.c_uint32)]


class PheError(RuntimeError):
    def __init__(self, status: int, where: str, text: str):
        super().__init__(f"{where}: status {status}: {text}")
        self.status = status


_VP = C.c_void_p
_U32 = C.c_uint32
_I32 = C.c_int
_F = C.c_float
_PF = C.POINTER(C.c_float)

# name -> (restype, argtypes); every function declared in include/phe_gb300.h
SIGNATURES: dict[str, tuple] = {
    "phe_version": (C.c_int, []),
    "phe_last_error": (C.c_char_p, []),
    "phe_scene_recipe_triangles": (C.c_uint64, [C.POINTER(SceneRecipe)]),
    "phe_scene_generate": (_I32, [C.POINTER(SceneRecipe), _VP, _VP, _VP]),
    "phe_sbvh_default_params": (None, [C.POINTER(SbvhParams)]),
    "phe_sbvh_build": (_I32, [_VP, _U32, C.POINTER(SbvhParams), C.POINTER(_VP)]),
    "phe_host_bvh_info": (_I32, [_VP, C.POINTER(_U32), C.POINTER(_U32), C.POINTER(_U32)]),
    "phe_host_bvh_copy": (_I32, [_VP, _VP, _VP, _VP]),
    "phe_host_bvh_free": (None, [_VP]),
    "phe_bvh_validate": (_I32, [_VP, _U32, _U32, C.POINTER(_U32)]),
    "phe_bvh_wide8_build": (_I32, [_VP, _U32, _U32, _VP, _U32, _VP, _U32, C.POINTER(_U32), C.POINTER(_U32),
                                   C.POINTER(_U32)]),
    "phe_bvh_cache_write": (_I32, [C.c_char_p, _VP, _U32, _VP, _VP, _U32]),
    "phe_bvh_cache_sizes": (_I32, [C.c_char_p, C.POINTER(_U32), C.POINTER(_U32)]),
    "phe_bvh_cache_read": (_I32, [C.c_char_p, _VP, _U32, _VP, _VP, _U32]),
    "phe_generate_camera_def": (None, [_PF, _PF, _PF, _F, _F, _F, C.POINTER(CameraDef)]),
    "phe_halton_jitter": (None, [_U32, _PF]),
    "phe_scene_create": (_I32, [_VP, _U32, _VP, _VP, _U32, _VP, _U32, _I32, C.POINTER(_VP)]),
    "phe_scene_set_materials_and_textures": (_I32, [_VP, _VP, _U32, C.POINTER(Texture), _U32]),
    "phe_scene_destroy": (_I32, [_VP]),
    "phe_scene_device_bytes": (_I32, [_VP, C.POINTER(C.c_uint64)]),
    "phe_cast_closest": (_I32, [_VP, _VP, _VP, _U32, _VP]),
    "phe_cast_closest_plain": (_I32, [_VP, _VP, _VP, _U32, _VP]),
    "phe_cast_any": (_I32, [_VP, _VP, _VP, _U32, _VP, _VP]),
    "phe_gen_primary_rays": (_I32, [_VP, C.POINTER(CameraDef), _U32, _U32, _F, _F, _I32, _VP]),
    "phe_scene_status": (_I32, [_VP, C.POINTER(_U32)]),
    "phe_scene_set_layout": (_I32, [_VP, _I32]),
    "phe_scene_get_layout": (_I32, [_VP, C.POINTER(_I32), C.POINTER(_I32)]),
    "phe_renderer_create": (_I32, [C.POINTER(_VP)]),
    "phe_renderer_destroy": (_I32, [_VP]),
    "phe_renderer_set_static_scene": (_I32, [_VP, _VP]),
    "phe_renderer_set_target_resolution": (_I32, [_VP, _U32, _U32]),
    "phe_renderer_update_camera": (_I32, [_VP, _PF, _PF, _PF, _F, _F, _F]),
    "phe_renderer_set_camera_def": (_I32, [_VP, C.POINTER(CameraDef), _PF, _F, _F]),
    "phe_renderer_set_seed": (_I32, [_VP, C.c_uint64, _U32]),
    "phe_renderer_set_graph": (_I32, [_VP, _I32]),
    "phe_renderer_reset_taa": (_I32, [_VP, _VP]),
    "phe_renderer_render": (_I32, [_VP, _VP, _U32, _VP]),
    "phe_renderer_result": (_I32, [_VP, C.POINTER(RenderResult)]),
    "phe_renderer_read": (_I32, [_VP, _I32, _VP, _VP]),
    "phe_renderer_ray_counts": (_I32, [_VP, C.POINTER(C.c_uint64), _VP]),
    "phe_renderer_set_kernel_timing": (_I32, [_VP, _I32]),
    "phe_renderer_frame_param_bytes": (_U32, []),
    "phe_renderer_kernel_times": (_I32, [_VP, C.POINTER(C.c_double), C.POINTER(_U32), C.POINTER(_U32)]),
    "phe_renderer_set_pipeline": (_I32, [_VP, _I32, _I32, _I32]),
    "phe_renderer_set_shadow_schedule": (_I32, [_VP, _I32]),
    "phe_renderer_read_async": (_I32, [_VP, _I32, _VP, _VP]),
    "phe_renderer_read_wait": (_I32, [_VP]),
    "phe_renderer_set_frames_in_flight": (_I32, [_VP, _I32]),
    "phe_renderer_set_frame_parts": (_I32, [_VP, _I32]),
    "phe_renderer_join": (_I32, [_VP, _VP]),
    "phe_renderer_set_latency_recording": (_I32, [_VP, _I32]),
    "phe_renderer_frame_latencies": (_I32, [_VP, _PF, _U32, C.POINTER(_U32)]),
    "phe_batch_default_params": (None, [C.POINTER(BatchParams)]),
    "phe_batch_create": (_I32, [C.POINTER(_VP), _U32, C.POINTER(BatchItem), _U32, C.POINTER(BatchParams), C.POINTER(_VP)]),
    "phe_batch_update": (_I32, [_VP, C.POINTER(BatchItem), _U32]),
    "phe_batch_set_params": (_I32, [_VP, C.POINTER(BatchParams)]),
    "phe_batch_launch": (_I32, [_VP, _VP]),
    "phe_batch_info": (_I32, [_VP, C.POINTER(C.c_uint64), C.POINTER(_U32)]),
    "phe_batch_autotune": (_I32, [_VP, _I32, _VP, C.POINTER(BatchParams), C.POINTER(C.c_float),
                                  C.POINTER(BatchTuningRow), _U32, C.POINTER(_U32)]),
    "phe_batch_destroy": (_I32, [_VP]),
    "phe_batch_cast_noalloc": (_I32, [C.POINTER(_VP), _U32, C.POINTER(BatchItem), _U32, _VP]),
    "phe_renderer_reset_ray_totals": (_I32, [_VP, _VP]),
    "phe_renderer_ray_totals_async": (_I32, [_VP, C.POINTER(C.c_uint64), _VP]),
    "phe_server_default_config": (None, [C.POINTER(ServerConfig)]),
    "phe_server_create": (_I32, [C.POINTER(ServerConfig), C.POINTER(_VP)]),
    "phe_server_add_scene": (_I32, [_VP, _VP, C.POINTER(_U32)]),
    "phe_server_submit": (_I32, [_VP, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "phe_server_poll": (_I32, [_VP, C.c_uint64, C.POINTER(RequestStats)]),
    "phe_server_wait": (_I32, [_VP, C.c_uint64, C.POINTER(RequestStats)]),
    "phe_server_drain": (_I32, [_VP]),
    "phe_server_release": (_I32, [_VP, C.c_uint64]),
    "phe_server_cancel": (_I32, [_VP, C.c_uint64]),
    "phe_server_get_stats": (_I32, [_VP, C.POINTER(ServerStats)]),
    "phe_server_destroy": (_I32, [_VP]),
    "phe_postprocess": (_I32, [_U32, _U32, _VP, _F, _VP, _VP, _VP]),
    "phe_scale": (_I32, [_U32, _U32, _VP, _U32, _U32, _U32, _U32, _VP, _VP, _VP]),
    "phe_taa_resolve": (_I32, [_U32, _U32, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
}

_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Loads libphe_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m phantasyenginetestbed_gb300.build"
                               f"{' --checked' if CHECKED else ''}`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != PHE_OK:
        raise PheError(status, where, lib().phe_last_error().decode(errors="replace"))


def ptr(a) -> int | None:
    """Raw address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")


def fvec(v) -> C.Array:
    a = (C.c_float * 3)(*[float(x) for x in v])
    return a
