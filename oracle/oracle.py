"""Test infrastructure only: ctypes wrappers of the oracle (oracle/liboracle.so) and, where it was
built from the reference sources, of the reference harness (oracle/_ref/libpheref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and reference legs may import this
module; it checks results and times the CPU baseline, and is never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "libpheref.so"
REF_SHADING_SO = HERE / "_ref" / "libpheref_shading.so"
# The reference files the harnesses compile: baseline/_ref, where oracle/stage_reference.py stages them
# (git-ignored; it travels with the repository), unless PHE_REFERENCE_ROOT names another tree.
REFERENCE_ROOT = Path(os.environ.get("PHE_REFERENCE_ROOT") or HERE.parent / "baseline" / "_ref")

MODE_CPU = 0   # castRay accept rule: t < closest && tMin <= t <= tMax (BVHTraversal.hpp:176)
MODE_GPU = 1   # rayCastKernel accept rule: tMin <= t < current (RayCastKernel.cu:361)

NODE_DTYPE = np.dtype([("fData", "<f4", (12,)), ("iData", "<i4", (4,))])
TRI_VERTS_DTYPE = np.dtype([("v0", "<f4", (4,)), ("v1", "<f4", (4,)), ("v2", "<f4", (4,))])
RAY_IN_DTYPE = np.dtype([("origin", "<f4", (3,)), ("tMin", "<f4"), ("dir", "<f4", (3,)), ("tMax", "<f4")])
RAY_HIT_DTYPE = np.dtype([("triangleIndex", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
LIGHT_DTYPE = np.dtype([("pos", "<f4", (3,)), ("radius", "<f4"), ("range", "<f4"), ("strength", "<f4", (3,)),
                        ("staticShadows", "<i4")])


class FrameParams(C.Structure):
    _fields_ = [("resX", C.c_uint32), ("resY", C.c_uint32), ("cam", C.c_float * 12), ("jitter", C.c_float * 2),
                ("camPos", C.c_float * 3), ("lights", C.c_void_p), ("numLights", C.c_uint32),
                ("materials", C.c_void_p), ("seed", C.c_uint64), ("frame", C.c_uint32),
                ("textures", C.c_void_p), ("numTextures", C.c_uint32), ("rowBegin", C.c_uint32),
                ("rowEnd", C.c_uint32), ("prevCam", C.c_float * 12), ("velocity", C.c_void_p),
                ("dump", C.c_void_p * 4), ("dumpCapacity", C.c_uint32 * 4), ("dumpCount", C.c_void_p)]


class Texture(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("bytesPerPixel", C.c_uint32),
                ("pitch", C.c_uint32)]


def textures_array(textures):
    """ctypes array of or_texture over (H, W, C) uint8 images (the images must stay alive)."""
    arr = (Texture * max(1, len(textures)))()
    for k, img in enumerate(textures):
        img3 = img.reshape(img.shape[0], img.shape[1], -1)
        assert img3.dtype == np.uint8 and img3.flags.c_contiguous
        arr[k] = Texture(img3.ctypes.data, img3.shape[1], img3.shape[0], img3.shape[2], img3.shape[1] * img3.shape[2])
    return arr


def scale(src, dst_res, viewport=None):
    """scaling.frag restated: (H, W, 4) float32 source -> (dstH, dstW, 4)."""
    src = np.ascontiguousarray(src, np.float32)
    H, W = src.shape[:2]
    vw, vh = viewport or (W, H)
    out = np.empty((dst_res[1], dst_res[0], 4), np.float32)
    lib().oracle_scale(W, H, _p(src), vw, vh, dst_res[0], dst_res[1], _p(out))
    return out


def texel_coord(c, n):
    return int(lib().oracle_texel_coord(C.c_float(c), n))


def srgb_table():
    out = np.empty(256, np.float32)
    lib().oracle_srgb_table(_p(out))
    return out


def build() -> None:
    """Builds liboracle.so, and the reference harnesses when the reference sources are present (staging
    them into baseline/_ref first when a reference checkout is at hand and they are not staged yet)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    if "PHE_REFERENCE_ROOT" not in os.environ:
        from oracle import stage_reference as S
        src = S.source_root()
        if src is not None and not S.staged():
            S.stage(src)
    if (REFERENCE_ROOT / "source").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REFERENCE_ROOT}"], check=True)


_o = None
_r = None


def _p(a):
    return None if a is None else a.ctypes.data


def lib():
    global _o
    if _o is None:
        if not ORACLE_SO.exists():
            build()
        L = C.CDLL(str(ORACLE_SO))
        V = C.c_void_p
        L.oracle_cast_rays.argtypes = [V, V, V, C.c_uint32, C.c_int, V, V, C.c_int]
        L.oracle_any_rays.argtypes = [V, V, V, C.c_uint32, V, C.c_int]
        L.oracle_brute_closest.argtypes = [V, C.c_uint32, V, C.c_uint32, C.c_int, V]
        L.oracle_brute_closest.restype = None
        L.oracle_intersect_tri.argtypes = [V, V, V, V, V, V]
        L.oracle_camera_def.argtypes = [V, V, V, C.c_float, C.c_float, C.c_float, V]
        L.oracle_camera_def.restype = None
        L.oracle_gen_primary.argtypes = [V, C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_int, V]
        L.oracle_gen_primary.restype = None
        L.oracle_render_frame.argtypes = [V, V, V, C.POINTER(FrameParams), V, V, V, V, V, C.c_int]
        L.oracle_taa.argtypes = [C.c_uint32, C.c_uint32, V, V, V, V, V, V, V]
        L.oracle_taa.restype = None
        L.oracle_postprocess.argtypes = [C.c_uint32, V, C.c_float, V]
        L.oracle_postprocess.restype = None
        L.oracle_halton_jitter.argtypes = [C.c_uint32, V]
        L.oracle_halton_jitter.restype = None
        L.oracle_sincos_2pi.argtypes = [C.c_float, V, V]
        L.oracle_sincos_2pi.restype = None
        L.oracle_scale.argtypes = [C.c_uint32, C.c_uint32, V, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, V]
        L.oracle_scale.restype = None
        L.oracle_texel_coord.argtypes = [C.c_float, C.c_int32]
        L.oracle_texel_coord.restype = C.c_uint32
        L.oracle_srgb_table.argtypes = [V]
        L.oracle_srgb_table.restype = None
        L.oracle_pixel_stream.argtypes = [V, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        L.oracle_pixel_stream.restype = None
        L.oracle_pcg_uniform.argtypes = [V]
        L.oracle_pcg_uniform.restype = C.c_float
        L.oracle_pcg_next.argtypes = [V]
        L.oracle_pcg_next.restype = C.c_uint32
        L.oracle_shade.argtypes = [V, V, V, V, C.c_float, C.c_float, V, C.c_float, V, C.c_float, V]
        L.oracle_shade.restype = None
        L.oracle_falloff.argtypes = [C.c_float, C.c_float]
        L.oracle_falloff.restype = C.c_float
        L.oracle_sample_lambert.argtypes = [C.c_float, C.c_float, V, V]
        L.oracle_sample_lambert.restype = None
        L.oracle_sample_ggx_bounce.argtypes = [C.c_float, C.c_float, C.c_float, V, V, V]
        L.oracle_sample_ggx_bounce.restype = None
        L.oracle_retrieve_tri_data.argtypes = [C.c_uint32, V, V, V, V, V]
        L.oracle_retrieve_tri_data.restype = None
        L.oracle_shade_hit.argtypes = [V, V, V, V, V, V, C.c_float, C.c_float, V, V, V]
        L.oracle_shade_hit.restype = C.c_int
        _o = L
    return _o


def ref_available() -> bool:
    return REF_SO.exists()


def ref_shading_available() -> bool:
    return REF_SHADING_SO.exists()


_rs = None


def ref_shading():
    """The reference's shading, sampling and hit-interpretation functions compiled as host code
    (oracle/ref_shading.cpp)."""
    global _rs
    if _rs is None:
        L = C.CDLL(str(REF_SHADING_SO))
        V = C.c_void_p
        for name, args in (("ref_shade", [C.c_uint32, V, V]), ("ref_falloff", [C.c_uint32, V, V, V]),
                           ("ref_sample_lambertian", [C.c_uint32, V, V]), ("ref_sample_ggx", [C.c_uint32, V, V]),
                           ("ref_retrieve_tri_data", [C.c_uint32, V, V, V, V, V]),
                           ("ref_shade_hit", [C.c_uint32, V, V, V, V])):
            getattr(L, name).argtypes = args
            getattr(L, name).restype = None
        _rs = L
    return _rs


def ref():
    global _r
    if _r is None:
        L = C.CDLL(str(REF_SO))
        V = C.c_void_p
        L.ref_build_sbvh.argtypes = [V, V, C.c_uint32]
        L.ref_build_sbvh.restype = V
        L.ref_bvh_sizes.argtypes = [V, V, V]
        L.ref_bvh_copy.argtypes = [V, V, V, V]
        L.ref_bvh_free.argtypes = [V]
        L.ref_cast_rays.argtypes = [V, V, V, C.c_uint32, V, V, C.c_int]
        L.ref_any_rays.argtypes = [V, V, V, C.c_uint32, V, C.c_int]
        L.ref_any_rays.restype = None
        L.ref_intersect_tri.argtypes = [V, V, V, V]
        L.ref_camera_def.argtypes = [V, V, V, C.c_float, C.c_float, C.c_float, V]
        _r = L
    return _r


def threads() -> int:
    return os.cpu_count() or 1


# ---------------------------------------------------------------------------------------------
# oracle

def cast_rays(nodes, verts, rays, mode=MODE_GPU, debug=False, nthreads=None):
    n = len(rays)
    hits = np.empty(n, RAY_HIT_DTYPE)
    dbg = np.empty((n, 2), np.uint32) if debug else None
    rc = lib().oracle_cast_rays(_p(nodes), _p(verts), _p(rays), n, mode, _p(hits), _p(dbg), nthreads or threads())
    if rc:
        raise RuntimeError(f"oracle: {rc} rays overflowed the traversal stack")
    return (hits, dbg) if debug else hits


def any_rays(nodes, verts, rays, nthreads=None):
    n = len(rays)
    out = np.empty(n, np.uint8)
    rc = lib().oracle_any_rays(_p(nodes), _p(verts), _p(rays), n, _p(out), nthreads or threads())
    if rc:
        raise RuntimeError(f"oracle: {rc} rays overflowed the traversal stack")
    return out


def brute_closest(tris, rays, mode=MODE_GPU):
    hits = np.empty(len(rays), RAY_HIT_DTYPE)
    lib().oracle_brute_closest(_p(tris), len(tris), _p(rays), len(rays), mode, _p(hits))
    return hits


def intersect_tri(tri_verts_row, origin, direction):
    tri = np.ascontiguousarray(tri_verts_row)
    o = np.asarray(origin, np.float32)
    d = np.asarray(direction, np.float32)
    t, u, v = (C.c_float(), C.c_float(), C.c_float())
    h = lib().oracle_intersect_tri(_p(tri), _p(o), _p(d), C.addressof(t), C.addressof(u), C.addressof(v))
    return bool(h), t.value, u.value, v.value


def camera_def(pos, direction, up, vfov_rad, res):
    out = np.empty(12, np.float32)
    a, b, c = (np.asarray(x, np.float32) for x in (pos, direction, up))
    lib().oracle_camera_def(_p(a), _p(b), _p(c), vfov_rad, float(res[0]), float(res[1]), _p(out))
    return out


def gen_primary(cam12, res, jitter=(0.0, 0.0), order=0):
    rays = np.empty(res[0] * res[1], RAY_IN_DTYPE)
    cam = np.ascontiguousarray(cam12, np.float32)
    lib().oracle_gen_primary(_p(cam), res[0], res[1], jitter[0], jitter[1], order, _p(rays))
    return rays


def halton_jitter(i):
    out = np.empty(2, np.float32)
    lib().oracle_halton_jitter(i, _p(out))
    return out


def sincos_2pi(r):
    s, c = C.c_float(), C.c_float()
    lib().oracle_sincos_2pi(r, C.addressof(s), C.addressof(c))
    return s.value, c.value


def render_frame(nodes, verts, slot_datas, materials, lights, cam12, res, jitter, cam_pos, seed, frame,
                 primary_hits=None, nthreads=None, work=None, textures=(), rows=None, prev_cam=None,
                 velocity_out=None, dump=None):
    """Oracle frame: (color (H, W, 4), roughness (H, W), ray counts per stage). `work` (optional
    uint64 array of 8) receives nodesVisited / triangle tests summed per stage; `textures` are
    (H, W, C) uint8 images indexed by the materials' texture indices; `rows` = (begin, end) renders
    only those rows (the rest of the image is left unset, the counts cover those rows); `velocity_out`
    ((H, W, 2) float32) receives the TAA velocity against the previous camera `prev_cam`; `dump` (a list
    of 4 RAY_IN_DTYPE arrays) receives the rays cast per stage (primary, primary shadow, bounce, bounce
    shadow), and is replaced by the filled prefixes."""
    fp = FrameParams()
    fp.resX, fp.resY = res
    fp.cam[:] = [float(x) for x in cam12]
    fp.jitter[:] = [float(jitter[0]), float(jitter[1])]
    fp.camPos[:] = [float(x) for x in cam_pos]
    lights = np.ascontiguousarray(lights, LIGHT_DTYPE)
    fp.lights = lights.ctypes.data
    fp.numLights = len(lights)
    fp.materials = materials.ctypes.data
    fp.seed = seed
    fp.frame = frame
    tex = textures_array(textures)
    fp.textures = C.addressof(tex)
    fp.numTextures = len(textures)
    if rows is not None:
        fp.rowBegin, fp.rowEnd = int(rows[0]), int(rows[1])
    if velocity_out is not None:
        assert velocity_out.dtype == np.float32 and velocity_out.shape == (res[1], res[0], 2)
        fp.prevCam[:] = [float(x) for x in (cam12 if prev_cam is None else prev_cam)]
        fp.velocity = velocity_out.ctypes.data
    dump_count = np.zeros(4, np.uint32)
    if dump is not None:
        for k in range(4):
            assert dump[k].dtype == RAY_IN_DTYPE and dump[k].flags.c_contiguous
            fp.dump[k] = dump[k].ctypes.data
            fp.dumpCapacity[k] = len(dump[k])
        fp.dumpCount = dump_count.ctypes.data
    color = np.empty((res[1], res[0], 4), np.float32)
    rough = np.empty((res[1], res[0]), np.float32)
    counts = np.zeros(4, np.uint64)
    rc = lib().oracle_render_frame(_p(nodes), _p(verts), _p(slot_datas), C.byref(fp), _p(primary_hits), _p(color),
                                   _p(rough), _p(counts), _p(work), nthreads or threads())
    if rc:
        raise RuntimeError(f"oracle: {rc} rays overflowed the traversal stack")
    if dump is not None:
        assert (dump_count <= np.array([len(d) for d in dump])).all(), "ray dump capacity exceeded"
        dump[:] = [d[:int(c)] for d, c in zip(dump, dump_count)]
    return color, rough, counts


def taa(cur, hist, roughness, velocity=None, prev_velocity=None):
    H, W = cur.shape[:2]
    out_c = np.empty_like(cur)
    out_h = np.empty_like(cur)
    lib().oracle_taa(W, H, _p(cur), _p(hist), _p(velocity), _p(prev_velocity), _p(roughness), _p(out_c), _p(out_h))
    return out_c, out_h


# ---------------------------------------------------------------------------------------------
# reference harness (only where oracle/_ref was built from the reference sources)

def ref_build_sbvh(tri_verts):
    tv = np.ascontiguousarray(tri_verts, np.float32).reshape(-1, 9)
    h = ref().ref_build_sbvh(_p(tv), None, tv.shape[0])
    nn, ns = C.c_uint32(), C.c_uint32()
    ref().ref_bvh_sizes(h, C.addressof(nn), C.addressof(ns))
    nodes = np.empty(nn.value, NODE_DTYPE)
    verts = np.empty(ns.value, TRI_VERTS_DTYPE)
    s2t = np.empty(ns.value, np.uint32)
    ref().ref_bvh_copy(h, _p(nodes), _p(verts), _p(s2t))
    ref().ref_bvh_free(h)
    return nodes, verts, s2t


def ref_cast_rays(nodes, verts, rays, debug=False, nthreads=None):
    n = len(rays)
    hits = np.empty(n, RAY_HIT_DTYPE)
    dbg = np.empty((n, 2), np.uint32) if debug else None
    ref().ref_cast_rays(_p(nodes), _p(verts), _p(rays), n, _p(hits), _p(dbg), nthreads or threads())
    return (hits, dbg) if debug else hits


def ref_any_rays(nodes, verts, rays, nthreads=None):
    """Any hit through the reference castRay: 1 where it finds no triangle in [tMin, tMax]."""
    out = np.empty(len(rays), np.uint8)
    ref().ref_any_rays(_p(nodes), _p(verts), _p(np.ascontiguousarray(rays, RAY_IN_DTYPE)), len(rays), _p(out),
                       nthreads or threads())
    return out


def ref_camera_def(pos, direction, up, vfov_rad, res):
    out = np.empty(12, np.float32)
    a, b, c = (np.asarray(x, np.float32) for x in (pos, direction, up))
    ref().ref_camera_def(_p(a), _p(b), _p(c), vfov_rad, float(res[0]), float(res[1]), _p(out))
    return out


# ---------------------------------------------------------------------------------------------
# comparison rule for closest-hit results

def compare_closest(test_hits, oracle_hits, rays, slot_to_tri, verts, rel_t=1e-6, rel_tuv=1e-5):
    """Compares closest-hit results under the parity rule: hit/miss identical; the original
    triangle identical with t, u, v within `rel_tuv` relative; or a documented near-tie — a different
    triangle whose t is within `rel_t` relative of the oracle's and which the oracle's own triangle
    test confirms at exactly the reported (t, u, v). Returns a dict of counts and the failing indices."""
    th, oh = test_hits, oracle_hits
    miss_t = th["triangleIndex"] == 0xFFFFFFFF
    miss_o = oh["triangleIndex"] == 0xFFFFFFFF
    flip = np.nonzero(miss_t != miss_o)[0]
    both = np.nonzero(~miss_t & ~miss_o)[0]
    ot = slot_to_tri[th["triangleIndex"][both]]
    oo = slot_to_tri[oh["triangleIndex"][both]]
    same = both[ot == oo]
    diff = both[ot != oo]
    bad_vals = []
    for k in ("t", "u", "v"):
        a = th[k][same].astype(np.float64)
        b = oh[k][same].astype(np.float64)
        tol = rel_tuv * np.maximum(np.abs(b), 1.0 if k != "t" else np.abs(b))
        bad = same[np.abs(a - b) > np.maximum(tol, 1e-30)]
        bad_vals.append(bad)
    bad_vals = np.unique(np.concatenate(bad_vals)) if bad_vals else np.array([], np.int64)
    near_ties, bad_ties = [], []
    for i in diff:
        tt, to = float(th["t"][i]), float(oh["t"][i])
        ok = abs(tt - to) <= rel_t * abs(to)
        if ok:
            r = rays[i]
            hit, t, u, v = intersect_tri(verts[th["triangleIndex"][i]], r["origin"], r["dir"])
            ok = hit and np.float32(t) == th["t"][i] and np.float32(u) == th["u"][i] and np.float32(v) == th["v"][i]
        (near_ties if ok else bad_ties).append(int(i))
    miss_vals = np.nonzero(miss_t & miss_o & (th["t"] != oh["t"]))[0]
    return {
        "rays": len(rays), "hits": int((~miss_o).sum()), "exact": int(len(same)) - len(bad_vals),
        "near_ties": len(near_ties), "hit_miss_flips": flip.tolist(), "bad_values": bad_vals.tolist(),
        "bad_ties": bad_ties, "miss_t_mismatch": miss_vals.tolist(),
        "ok": len(flip) == 0 and len(bad_vals) == 0 and len(bad_ties) == 0 and len(miss_vals) == 0,
    }


def postprocess(linear, gamma=2.2):
    lin = np.ascontiguousarray(linear, np.float32)
    out = np.empty_like(lin)
    lib().oracle_postprocess(lin.size // 4, _p(lin), gamma, _p(out))
    return out


# ---------------------------------------------------------------------------------------------
# shading, sampling and hit interpretation on rows of inputs: the oracle (left) and the reference's
# own functions (ref_*, oracle/ref_shading.cpp) take the same row layouts
#   shade:      22 floats  p.xyz n.xyz v.xyz albedo.rgb roughness metallic l.xyz toLightDist strength.rgb range
#   lambert:     5 floats  r1 r2 n.xyz
#   ggx:         9 floats  r1 r2 roughness fromCamera.xyz n.xyz
#   shade_hit:  28 floats  mask.rgb n.xyz toCamera.xyz pos.xyz albedo.rgb metallic roughness
#                          light.pos.xyz light.radius light.range light.strength.rgb light.staticShadows r1 r2

TRI_DATA_DTYPE = np.dtype([("n0", "<f4", (3,)), ("n1", "<f4", (3,)), ("n2", "<f4", (3,)), ("uv0", "<f4", (2,)),
                           ("uv1", "<f4", (2,)), ("uv2", "<f4", (2,)), ("materialIndex", "<u4")])


def _rows(a, width):
    a = np.ascontiguousarray(a, np.float32)
    assert a.ndim == 2 and a.shape[1] == width
    return a


def shade_rows(rows):
    rows = _rows(rows, 22)
    out = np.empty((len(rows), 3), np.float32)
    L = lib()
    for i, r in enumerate(rows):
        L.oracle_shade(_p(r[0:3]), _p(r[3:6]), _p(r[6:9]), _p(r[9:12]), float(r[12]), float(r[13]), _p(r[14:17]),
                       float(r[17]), _p(r[18:21]), float(r[21]), _p(out[i]))
    return out


def falloff_rows(dist, rng):
    return np.array([lib().oracle_falloff(float(d), float(r)) for d, r in zip(dist, rng)], np.float32)


def lambert_rows(rows):
    rows = _rows(rows, 5)
    out = np.empty((len(rows), 3), np.float32)
    for i, r in enumerate(rows):
        lib().oracle_sample_lambert(float(r[0]), float(r[1]), _p(r[2:5]), _p(out[i]))
    return out


def ggx_rows(rows):
    rows = _rows(rows, 9)
    out = np.empty((len(rows), 3), np.float32)
    for i, r in enumerate(rows):
        lib().oracle_sample_ggx_bounce(float(r[0]), float(r[1]), float(r[2]), _p(r[3:6]), _p(r[6:9]), _p(out[i]))
    return out


def retrieve_tri_data(datas, rays, hits):
    datas = np.ascontiguousarray(datas, TRI_DATA_DTYPE)
    rays = np.ascontiguousarray(rays, RAY_IN_DTYPE)
    hits = np.ascontiguousarray(hits, RAY_HIT_DTYPE)
    out = np.empty((len(datas), 8), np.float32)
    mat = np.empty(len(datas), np.uint32)
    lib().oracle_retrieve_tri_data(len(datas), _p(datas), _p(rays), _p(hits), _p(out), _p(mat))
    return out, mat


def shade_hit_rows(rows):
    rows = _rows(rows, 28)
    contrib = np.empty((len(rows), 3), np.float32)
    rays = np.zeros((len(rows), 8), np.float32)
    cast = np.empty(len(rows), np.uint8)
    light = np.zeros(1, LIGHT_DTYPE)
    L = lib()
    for i, r in enumerate(rows):
        light["pos"] = r[17:20]
        light["radius"] = r[20]
        light["range"] = r[21]
        light["strength"] = r[22:25]
        light["staticShadows"] = int(r[25] != 0)
        cast[i] = L.oracle_shade_hit(_p(light), _p(r[0:3]), _p(r[3:6]), _p(r[6:9]), _p(r[9:12]), _p(r[12:15]),
                                     float(r[15]), float(r[16]), _p(r[26:28]), _p(contrib[i]), _p(rays[i]))
    return contrib, rays, cast


def ref_shade_rows(rows):
    rows = _rows(rows, 22)
    out = np.empty((len(rows), 3), np.float32)
    ref_shading().ref_shade(len(rows), _p(rows), _p(out))
    return out


def ref_falloff_rows(dist, rng):
    dist = np.ascontiguousarray(dist, np.float32)
    rng = np.ascontiguousarray(rng, np.float32)
    out = np.empty(len(dist), np.float32)
    ref_shading().ref_falloff(len(dist), _p(dist), _p(rng), _p(out))
    return out


def ref_lambert_rows(rows):
    rows = _rows(rows, 5)
    out = np.empty((len(rows), 3), np.float32)
    ref_shading().ref_sample_lambertian(len(rows), _p(rows), _p(out))
    return out


def ref_ggx_rows(rows):
    rows = _rows(rows, 9)
    out = np.empty((len(rows), 3), np.float32)
    ref_shading().ref_sample_ggx(len(rows), _p(rows), _p(out))
    return out


def ref_retrieve_tri_data(datas, rays, hits):
    datas = np.ascontiguousarray(datas, TRI_DATA_DTYPE)
    rays = np.ascontiguousarray(rays, RAY_IN_DTYPE)
    hits = np.ascontiguousarray(hits, RAY_HIT_DTYPE)
    out = np.empty((len(datas), 8), np.float32)
    mat = np.empty(len(datas), np.uint32)
    ref_shading().ref_retrieve_tri_data(len(datas), _p(datas), _p(rays), _p(hits), _p(out), _p(mat))
    return out, mat


def ref_shade_hit_rows(rows):
    rows = _rows(rows, 28)
    contrib = np.empty((len(rows), 3), np.float32)
    rays = np.empty((len(rows), 8), np.float32)
    cast = np.empty(len(rows), np.uint8)
    ref_shading().ref_shade_hit(len(rows), _p(rows), _p(contrib), _p(rays), _p(cast))
    return contrib, rays, cast
