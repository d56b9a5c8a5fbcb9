"""Shared test helpers: scenes, reconstruction of slot vertices from a slot map, device buffers."""
from __future__ import annotations

import math
from functools import lru_cache
from pathlib import Path

import numpy as np

import phantasyenginetestbed_gb300 as P
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
C1_CAM = dict(pos=(0.5, -0.3, 0.6), dir=(0.0, 0.8, -0.6), up=(0.0, 0.6, 0.8), vfov=60.0, res=(512, 512))


def slot_verts(nodes: np.ndarray, slot_to_tri: np.ndarray, tri_verts: np.ndarray) -> np.ndarray:
    """TriangleVertices per slot with the sanitizeBVH end markers (-1 on each leaf's last slot)."""
    out = np.zeros(len(slot_to_tri), P.TRI_VERTS_DTYPE)
    tv = tri_verts[slot_to_tri]
    out["v0"][:, :3] = tv[:, 0:3]
    out["v1"][:, :3] = tv[:, 3:6]
    out["v2"][:, :3] = tv[:, 6:9]
    idx = nodes["iData"]
    for c in (0, 1):
        leaf = idx[:, 2 + c] > 0
        raw = idx[leaf, c]
        first = np.where(raw < 0, ~raw, raw)
        last = first + idx[leaf, 2 + c] - 1
        for k in ("v0", "v1", "v2"):
            out[k][last, 3] = -1.0
    return out


def load_golden(name: str):
    return np.load(GOLDEN / name, allow_pickle=False)


@lru_cache(maxsize=None)
def golden_scene(name: str):
    """(scene arrays, reference nodes, reference slot verts, slot map) of a golden fixture."""
    g = load_golden(name)
    grid, cubes, rot, seed = (int(x) for x in g["scene"])
    s = P.generate_scene(grid, cubes, bool(rot), seed)
    import hashlib
    digest = hashlib.sha256(np.ascontiguousarray(s.tri_verts).tobytes()).hexdigest()
    assert digest == str(g["digest"]), "scene generator output differs from the fixture's scene"
    nodes = g["nodes"]
    s2t = g["slot_to_tri"]
    verts = slot_verts(nodes, s2t, s.tri_verts)
    return s, nodes, verts, s2t


class RefTree:
    """A BVH built by the reference's own builder (buildStaticFrom + sanitizeBVH, compiled from the
    reference sources into oracle/_ref/libpheref.so), with the slot -> input-triangle map."""

    def __init__(self, nodes, verts, slot_to_tri):
        self.nodes, self.verts, self.slot_to_tri = nodes, verts, slot_to_tri

    def slot_datas(self, datas: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(datas[self.slot_to_tri])


@lru_cache(maxsize=None)
def ref_built_scene(name: str):
    """(scene arrays, RefTree) of a standard scene, built by the reference builder."""
    s = P.standard_scene(name)
    nodes, verts, s2t = O.ref_build_sbvh(s.tri_verts)
    return s, RefTree(nodes, verts, s2t)


@lru_cache(maxsize=None)
def built_scene(name: str):
    """(scene arrays, HostBVH from the project's builder) of a standard scene."""
    s = P.standard_scene(name)
    return s, P.build_sbvh(s.tri_verts)


def c1_camera():
    g = load_golden("ref_c1.npz")
    return g["cam"]


def cam_struct(cam12) -> P.CameraDef:
    c = P.CameraDef()
    c.origin[:] = [float(x) for x in cam12[0:3]]
    c.dir[:] = [float(x) for x in cam12[3:6]]
    c.dX[:] = [float(x) for x in cam12[6:9]]
    c.dY[:] = [float(x) for x in cam12[9:12]]
    return c


def random_rays(n: int, lo, hi, seed: int, tmin=1e-4, tmax=3.4028235e38) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, P.RAY_IN_DTYPE)
    rays["origin"] = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["dir"] = d.astype(np.float32)
    rays["tMin"] = np.float32(tmin)
    rays["tMax"] = np.float32(tmax)
    return rays


def hemisphere_rays_from_hits(rays: np.ndarray, hits: np.ndarray, tri_normals_of_slot, seed: int) -> np.ndarray:
    """Cosine-ish bounce rays from the hit points of `hits` (incoherent secondary rays)."""
    m = hits["triangleIndex"] != 0xFFFFFFFF
    r = rays[m]
    h = hits[m]
    pos = r["origin"] + r["dir"] * h["t"][:, None]
    n = tri_normals_of_slot(h["triangleIndex"])
    rng = np.random.default_rng(seed)
    d = rng.normal(size=pos.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = np.where((d * n).sum(1, keepdims=True) < 0, -d, d)
    out = np.zeros(len(pos), P.RAY_IN_DTYPE)
    out["origin"] = pos.astype(np.float32)
    out["dir"] = d.astype(np.float32)
    out["tMin"] = np.float32(1e-3)
    out["tMax"] = np.float32(3.4028235e38)
    return out


# --- device helpers (torch supplies memory only) ---------------------------------------------------

def to_device(a: np.ndarray):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()
    return t


def from_device(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(dtype)


def device_empty(n: int, dtype):
    import torch
    return torch.empty(n * np.dtype(dtype).itemsize, dtype=torch.uint8, device="cuda")


# --- seeded inputs for the shading comparison against the reference's own functions ---------------

def _unit(rng, n):
    d = rng.normal(size=(n, 3))
    return (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


def shading_inputs(n: int, seed: int) -> dict:
    """Rows for shade / falloff / sampleLambertian / sampleGgx / retrieveTriData / shadeHit in the layouts
    of oracle.oracle's *_rows functions. Includes the edge cases of each function: lights behind the
    surface and beyond their range, l = -v (a zero half vector), roughness and metallic at 0 and 1,
    normals within 0.001 of +-z (the other up vector), point and sphere lights, shadows off."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    out = {}
    nrm = _unit(rng, n)
    v = _unit(rng, n)
    l = _unit(rng, n)
    l[::97] = -v[::97]
    rough = rng.uniform(0, 1, n).astype(f32)
    rough[::11] = 0.0
    rough[5::11] = 1.0
    metal = rng.uniform(0, 1, n).astype(f32)
    metal[::7] = 0.0
    metal[3::7] = 1.0
    rngs = rng.uniform(0.5, 4.0, n).astype(f32)
    dist = (rngs * rng.uniform(0.01, 1.3, n)).astype(f32)
    shade = np.concatenate([rng.uniform(-2, 2, (n, 3)), nrm, v, rng.uniform(0, 1, (n, 3)), rough[:, None],
                            metal[:, None], l, dist[:, None], rng.uniform(0, 10, (n, 3)), rngs[:, None]], axis=1)
    out["shade"] = shade.astype(f32)
    out["falloff"] = np.stack([dist, rngs], axis=1)
    zn = _unit(rng, n)
    zn[::5] = np.array([0.0, 0.0, 1.0], f32)
    zn[1::5] = np.array([0.0, 0.0, -1.0], f32)
    zn[2::5, 2] = np.sign(zn[2::5, 2]) * rng.uniform(0.998, 1.0, len(zn[2::5])).astype(f32)
    zn = (zn / np.linalg.norm(zn, axis=1, keepdims=True)).astype(f32)
    r12 = rng.uniform(0, 1, (n, 2)).astype(f32)
    out["lambert"] = np.concatenate([r12, zn], axis=1).astype(f32)
    out["ggx"] = np.concatenate([r12, rough[:, None], _unit(rng, n), zn], axis=1).astype(f32)
    datas = np.zeros(n, P.TRI_DATA_DTYPE)
    for k in ("n0", "n1", "n2"):
        datas[k] = rng.normal(size=(n, 3)).astype(f32)
    for k in ("uv0", "uv1", "uv2"):
        datas[k] = rng.uniform(-2, 2, (n, 2)).astype(f32)
    datas["materialIndex"] = rng.integers(0, 1 << 20, n).astype(np.uint32)
    rays = np.zeros(n, P.RAY_IN_DTYPE)
    rays["origin"] = rng.uniform(-4, 4, (n, 3)).astype(f32)
    rays["dir"] = _unit(rng, n)
    hits = np.zeros(n, P.RAY_HIT_DTYPE)
    hits["t"] = rng.uniform(0, 10, n).astype(f32)
    uu = rng.uniform(0, 1, n)
    vv = rng.uniform(0, 1, n) * (1 - uu)
    hits["u"], hits["v"] = uu.astype(f32), vv.astype(f32)
    out["tri_data"] = (datas, rays, hits)
    pos = rng.uniform(0, 2, (n, 3)).astype(f32)
    lpos = (pos + rng.uniform(-2, 2, (n, 3))).astype(f32)
    radius = np.where(rng.uniform(size=n) < 0.5, 0.0, rng.uniform(0, 0.5, n)).astype(f32)
    shadows = (rng.uniform(size=n) < 0.85).astype(f32)
    out["shade_hit"] = np.concatenate(
        [rng.uniform(0, 1, (n, 3)), nrm, v, pos, rng.uniform(0, 1, (n, 3)), metal[:, None], rough[:, None], lpos,
         radius[:, None], rng.uniform(0.5, 4.0, (n, 1)), rng.uniform(0, 10, (n, 3)), shadows[:, None], r12],
        axis=1).astype(f32)
    return out
