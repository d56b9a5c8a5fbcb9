"""GB300-native ray-cast and wavefront-shading core, a drop-in for the ray-cast path of
PetorSFZ/PhantasyEngineTestbed.

Host API over the C ABI of libphe_gb300.so (include/phe_gb300.h):

* scene tools (host): :func:`generate_scene`, :func:`build_sbvh`, :func:`camera_def`, :func:`halton_jitter`
* device scenes: :class:`Scene` (``setStaticScene``, CudaTracerRenderer.cpp:251-315)
* ray casting: :func:`cast_closest`, :func:`cast_closest_plain`, :func:`cast_any`, :func:`gen_primary_rays`
* the reference's renderer: :class:`phantasyenginetestbed_gb300.renderer.CudaTracerRenderer`

Device buffers are torch CUDA tensors (or raw device addresses); torch supplies memory and streams
only, every computation runs in the library's CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

# Hardware work queues between the host and the GPU (read when the CUDA context is created; a value the
# process already set is kept). The serving loop runs a stream per render slot beside its query waves:
# with the default of 8 queues those streams share queues and wait on each other, and 32 gave 5% more
# served rays/s (4,905 vs 4,669 Mrays/s at 8,000 req/s); single-stream work is unaffected.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np

from . import native as _n
from .native import (LIGHT_DTYPE, MATERIAL_DTYPE, NODE_DTYPE, RAY_HIT_DTYPE, RAY_IN_DTYPE, TRI_DATA_DTYPE,
                     TRI_VERTS_DTYPE, CameraDef, PheError, check, lib, ptr)

__all__ = [
    "CameraDef", "PheError", "Scene", "HostBVH", "SceneArrays", "generate_scene", "build_sbvh", "camera_def",
    "halton_jitter", "wide8_build", "write_bvh_cache", "read_bvh_cache", "cast_closest", "cast_closest_plain", "cast_any", "gen_primary_rays", "STANDARD_SCENES",
    "NODE_DTYPE", "TRI_VERTS_DTYPE", "TRI_DATA_DTYPE", "RAY_IN_DTYPE", "RAY_HIT_DTYPE", "MATERIAL_DTYPE", "LIGHT_DTYPE",
]

# Scene recipes of the benchmark configurations: (grid cells N, cubes, rotated cubes, seed). The
# world is scaled by N/64 (cell size 1/64) so that the reference's absolute 1e-5 determinant
# epsilon (Intersection.hpp:28) stays far below the triangle scale.
STANDARD_SCENES = {
    "c1_64_100": (64, 100, False, 1),          # 9,392 triangles: plain closest-hit primary rays
    "c2_256_2000": (256, 2000, True, 2),       # 155,072 triangles: wavefront frame
    "c3_10k": (64, 150, False, 31),            # 9,992
    "c3_155k": (256, 2000, False, 32),         # 155,072
    "c3_1m": (724, 100, False, 33),            # 1,049,552
    "c3_2m": (1024, 100, False, 34),           # 2,098,352
    "c4_2048_20000": (2048, 20000, False, 4),  # 8,628,608: large incoherent workload
}


@dataclass
class SceneArrays:
    """A generated triangle soup: vertices (T, 9) float32, TriangleData and per-triangle materials."""
    tri_verts: np.ndarray
    datas: np.ndarray
    materials: np.ndarray
    scale: float


def generate_scene(grid: int, cubes: int, rotated: bool, seed: int, with_datas: bool = True) -> SceneArrays:
    """Seeded heightfield + cubes scene (phe_scene_generate)."""
    r = _n.SceneRecipe(grid, cubes, 1 if rotated else 0, 0, seed)
    T = int(lib().phe_scene_recipe_triangles(C.byref(r)))
    verts = np.empty((T, 9), np.float32)
    datas = np.empty(T, TRI_DATA_DTYPE) if with_datas else None
    mats = np.empty(T, MATERIAL_DTYPE) if with_datas else None
    check(lib().phe_scene_generate(C.byref(r), ptr(verts), ptr(datas), ptr(mats)), "phe_scene_generate")
    return SceneArrays(verts, datas, mats, grid / 64.0)


def standard_scene(name: str, with_datas: bool = True) -> SceneArrays:
    g, c, rot, seed = STANDARD_SCENES[name]
    return generate_scene(g, c, rot, seed, with_datas)


@dataclass
class HostBVH:
    """A BVH in the reference layout: nodes, slot vertices (with end markers), slot -> triangle map."""
    nodes: np.ndarray
    verts: np.ndarray
    slot_to_tri: np.ndarray
    max_depth: int

    def slot_datas(self, datas: np.ndarray) -> np.ndarray:
        """TriangleData per slot (duplicates are copies, StaticBVHBuilder.cpp:242-245)."""
        return datas[self.slot_to_tri]


def build_sbvh(tri_verts: np.ndarray, threads: int = 0, split_alpha: float = 1e-5) -> HostBVH:
    """Spatial-split BVH in the sanitized reference layout (phe_sbvh_build)."""
    tv = np.ascontiguousarray(tri_verts, np.float32).reshape(-1, 9)
    p = _n.SbvhParams()
    lib().phe_sbvh_default_params(C.byref(p))
    p.numThreads = threads
    p.splitAlpha = split_alpha
    h = C.c_void_p()
    check(lib().phe_sbvh_build(ptr(tv), tv.shape[0], C.byref(p), C.byref(h)), "phe_sbvh_build")
    try:
        nn, ns, md = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().phe_host_bvh_info(h, C.byref(nn), C.byref(ns), C.byref(md)), "phe_host_bvh_info")
        nodes = np.empty(nn.value, NODE_DTYPE)
        verts = np.empty(ns.value, TRI_VERTS_DTYPE)
        s2t = np.empty(ns.value, np.uint32)
        check(lib().phe_host_bvh_copy(h, ptr(nodes), ptr(verts), ptr(s2t)), "phe_host_bvh_copy")
    finally:
        lib().phe_host_bvh_free(h)
    return HostBVH(nodes, verts, s2t, int(md.value))


def write_bvh_cache(base: str, bvh: HostBVH, slot_datas: np.ndarray) -> None:
    """The reference's three-file BVH cache (Main.cpp:105-154) plus a checksummed header file."""
    datas = np.ascontiguousarray(slot_datas)
    assert datas.dtype == TRI_DATA_DTYPE and len(datas) == len(bvh.verts)
    check(lib().phe_bvh_cache_write(str(base).encode(), ptr(bvh.nodes), len(bvh.nodes), ptr(bvh.verts), ptr(datas),
                                    len(bvh.verts)), "phe_bvh_cache_write")


def read_bvh_cache(base: str):
    """(nodes, slot vertices, slot datas) of a cache; verified against its header when it has one."""
    nn, ns = C.c_uint32(), C.c_uint32()
    b = str(base).encode()
    check(lib().phe_bvh_cache_sizes(b, C.byref(nn), C.byref(ns)), "phe_bvh_cache_sizes")
    nodes = np.empty(nn.value, NODE_DTYPE)
    verts = np.empty(ns.value, TRI_VERTS_DTYPE)
    datas = np.empty(ns.value, TRI_DATA_DTYPE)
    check(lib().phe_bvh_cache_read(b, ptr(nodes), nn.value, ptr(verts), ptr(datas), ns.value), "phe_bvh_cache_read")
    return nodes, verts, datas


def validate_bvh(nodes: np.ndarray, num_slots: int) -> int:
    md = C.c_uint32()
    check(lib().phe_bvh_validate(ptr(nodes), len(nodes), num_slots, C.byref(md)), "phe_bvh_validate")
    return int(md.value)


def wide8_build(nodes: np.ndarray, num_slots: int):
    """The 8-wide compressed layout scene upload builds from a tree (phe_bvh_wide8_build): (node words
    (N, 20) uint32, leaf records (L, 8) uint32, depth)."""
    nodes = np.ascontiguousarray(nodes)
    nn, nl, dp = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(lib().phe_bvh_wide8_build(ptr(nodes), len(nodes), num_slots, None, 0, None, 0, C.byref(nn), C.byref(nl),
                                    C.byref(dp)), "phe_bvh_wide8_build")
    w = np.empty((nn.value, 20), np.uint32)
    lv = np.empty((nl.value, 8), np.uint32)
    check(lib().phe_bvh_wide8_build(ptr(nodes), len(nodes), num_slots, ptr(w), nn.value, ptr(lv), nl.value,
                                    C.byref(nn), C.byref(nl), C.byref(dp)), "phe_bvh_wide8_build")
    return w, lv, int(dp.value)


def camera_def(pos, direction, up, vfov_deg: float, res) -> CameraDef:
    """generateCameraDef (GenerateRays.cpp:12-35)."""
    out = CameraDef()
    lib().phe_generate_camera_def(_n.fvec(pos), _n.fvec(direction), _n.fvec(up), C.c_float(vfov_deg * math.pi / 180.0),
                                  C.c_float(res[0]), C.c_float(res[1]), C.byref(out))
    return out


def camera_def_array(cam: CameraDef) -> np.ndarray:
    return np.array(list(cam.origin) + list(cam.dir) + list(cam.dX) + list(cam.dY), np.float32)


def halton_jitter(i: int) -> tuple[float, float]:
    out = (C.c_float * 2)()
    lib().phe_halton_jitter(i, out)
    return float(out[0]), float(out[1])


class Scene:
    """A scene resident on the current CUDA device (phe_scene_create)."""

    def __init__(self, nodes: np.ndarray, verts: np.ndarray, datas: np.ndarray | None = None,
                 materials: np.ndarray | None = None):
        nodes = np.ascontiguousarray(nodes)
        verts = np.ascontiguousarray(verts)
        assert nodes.dtype == NODE_DTYPE and verts.dtype == TRI_VERTS_DTYPE
        if datas is not None:
            datas = np.ascontiguousarray(datas)
            assert datas.dtype == TRI_DATA_DTYPE and len(datas) == len(verts)
        if materials is not None:
            materials = np.ascontiguousarray(materials)
            assert materials.dtype == MATERIAL_DTYPE
        h = C.c_void_p()
        check(lib().phe_scene_create(ptr(nodes), len(nodes), ptr(verts), ptr(datas), len(verts), ptr(materials),
                                     0 if materials is None else len(materials), _n.PTR_HOST, C.byref(h)),
              "phe_scene_create")
        self.handle = h
        self.num_nodes = len(nodes)
        self.num_slots = len(verts)

    @classmethod
    def from_bvh(cls, bvh: HostBVH, scene: SceneArrays | None = None) -> "Scene":
        if scene is None:
            return cls(bvh.nodes, bvh.verts)
        return cls(bvh.nodes, bvh.verts, bvh.slot_datas(scene.datas), scene.materials)

    def setMaterialsAndTextures(self, materials: np.ndarray, textures=()) -> None:
        """setMaterialsAndTextures (CudaTracerRenderer.cpp:192-239): `materials` MATERIAL_DTYPE,
        `textures` (H, W[, C]) uint8 images with C in {1, 2, 4} (RawImage rows, row 0 first)."""
        materials = np.ascontiguousarray(materials)
        assert materials.dtype == MATERIAL_DTYPE
        imgs = [np.ascontiguousarray(t, np.uint8) for t in textures]
        arr = (_n.Texture * max(1, len(imgs)))()
        for k, img in enumerate(imgs):
            img3 = img.reshape(img.shape[0], img.shape[1], -1)
            arr[k] = _n.Texture(img3.ctypes.data, img3.shape[1], img3.shape[0], img3.shape[2],
                                img3.shape[1] * img3.shape[2])
        check(lib().phe_scene_set_materials_and_textures(self.handle, ptr(materials), len(materials), arr, len(imgs)),
              "phe_scene_set_materials_and_textures")

    def set_layout(self, layout: int) -> None:
        """0 = binary nodes (default), 1 = 4-wide nodes, 2 = 8-wide compressed nodes (same results; see
        phe_scene_set_layout)."""
        check(lib().phe_scene_set_layout(self.handle, layout), "phe_scene_set_layout")

    def layout(self):
        """(selected layout, mask of the wide layouts the tree allows: 1 = 4-wide, 2 = 8-wide)."""
        lay, avail = C.c_int(), C.c_int()
        check(lib().phe_scene_get_layout(self.handle, C.byref(lay), C.byref(avail)), "phe_scene_get_layout")
        return int(lay.value), int(avail.value)

    def status(self) -> int:
        """Error bits raised by kernels on this scene so far (1 = traversal stack overflow, 2 = index
        outside its array, which only the checked build tests); 0 when every traversal was sound."""
        bits = C.c_uint32()
        check(lib().phe_scene_status(self.handle, C.byref(bits)), "phe_scene_status")
        return int(bits.value)

    def device_bytes(self) -> int:
        b = C.c_uint64()
        check(lib().phe_scene_device_bytes(self.handle, C.byref(b)), "phe_scene_device_bytes")
        return int(b.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            check(lib().phe_scene_destroy(self.handle), "phe_scene_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def cast_closest(scene: Scene, rays, hits, n: int | None = None, stream=None) -> None:
    """Closest hit, persistent kernel (asynchronous on `stream`)."""
    n = rays.numel() * rays.element_size() // 32 if n is None else n
    check(lib().phe_cast_closest(scene.handle, ptr(rays), ptr(hits), n, _stream(stream)), "phe_cast_closest")


def cast_closest_plain(scene: Scene, rays, hits, n: int | None = None, stream=None) -> None:
    """Closest hit, one ray per thread (asynchronous on `stream`)."""
    n = rays.numel() * rays.element_size() // 32 if n is None else n
    check(lib().phe_cast_closest_plain(scene.handle, ptr(rays), ptr(hits), n, _stream(stream)), "phe_cast_closest_plain")


def cast_any(scene: Scene, rays, in_light, n: int | None = None, scatter=None, stream=None) -> None:
    """Any hit: in_light[i] = 1 when unoccluded in [tMin, tMax) (asynchronous on `stream`)."""
    n = rays.numel() * rays.element_size() // 32 if n is None else n
    check(lib().phe_cast_any(scene.handle, ptr(rays), ptr(in_light), n, ptr(scatter), _stream(stream)), "phe_cast_any")


def gen_primary_rays(rays, cam: CameraDef, res, jitter=(0.0, 0.0), order: int = 0, stream=None) -> None:
    check(lib().phe_gen_primary_rays(ptr(rays), C.byref(cam), int(res[0]), int(res[1]), C.c_float(jitter[0]),
                                     C.c_float(jitter[1]), order, _stream(stream)), "phe_gen_primary_rays")
