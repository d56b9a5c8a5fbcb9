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
