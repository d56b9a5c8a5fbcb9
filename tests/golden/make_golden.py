"""Generates the golden fixtures in tests/golden/ from the reference's own CPU code.

Needs the reference sources (staged into baseline/_ref by oracle/stage_reference.py, or the tree
named by PHE_REFERENCE_ROOT) to build oracle/_ref/libpheref.so, a harness around the reference's buildStaticFrom + sanitizeBVH, castRay /
castDebugRay, the triangle test and generateCameraDef. Inputs come from the project's seeded scene
generator and the oracle's primary-ray generator, both of which are deterministic across platforms.

Fixtures (npz, compressed):
  ref_small.npz   a 16x16-cell heightfield + 6 cubes: reference SBVH, 64x64 primary rays, all hits
  ref_c1.npz      the 64x64-cell + 100 cube scene of the plain closest-hit configuration: reference
                  SBVH (nodes + slot map), camera def, hits and traversal counters for every 16th of
                  the 512x512 primary rays, and 4096 incoherent rays with their hits
  ref_isect.npz   2000 ray/triangle pairs through the reference triangle test
  ref_halton.npy  the reference's 16-entry Halton table parsed from GameScreen.cpp
  ref_shading.npz 4096 input rows each through the reference's own shade, falloffFactor,
                  sampleLambertian, sampleGgx (as the bounce calls it), retrieveTriData and shadeHit
                  (oracle/_ref/libpheref_shading.so, the functions compiled as host code), with outputs

Run:  python tests/golden/make_golden.py [--only shading]
"""
from __future__ import annotations

import hashlib
import math
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[0] = str(ROOT)

import phantasyenginetestbed_gb300 as P  # noqa: E402
from oracle import oracle as O  # noqa: E402

C1_CAM = dict(pos=(0.5, -0.3, 0.6), dir=(0.0, 0.8, -0.6), up=(0.0, 0.6, 0.8), vfov=60.0, res=(512, 512))


def scene_digest(tri_verts: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(tri_verts, np.float32).tobytes()).hexdigest()


def incoherent_rays(scene_scale: float, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, O.RAY_IN_DTYPE)
    o = rng.uniform([0.0, 0.0, 0.05], [1.0, 1.0, 0.4], size=(n, 3)) * np.float32(scene_scale)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["origin"] = o.astype(np.float32)
    rays["dir"] = d.astype(np.float32)
    rays["tMin"] = np.float32(1e-4)
    rays["tMax"] = np.float32(3.4028235e38)
    return rays


def shading_digest(x: dict) -> str:
    """sha256 over every input row of the shading fixture (the test regenerates them and compares)."""
    h = hashlib.sha256()
    for k in ("shade", "falloff", "lambert", "ggx", "shade_hit"):
        h.update(np.ascontiguousarray(x[k]).tobytes())
    for a in x["tri_data"]:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def shading() -> None:
    """Reference outputs of the shading functions on the seeded rows of tests.helpers.shading_inputs."""
    from tests.helpers import shading_inputs
    if not O.ref_shading_available():
        raise SystemExit("reference shading harness not built: the reference sources are needed")
    x = shading_inputs(4096, 7)
    d, r, h = x["tri_data"]
    td, tm = O.ref_retrieve_tri_data(d, r, h)
    hc, hr, hk = O.ref_shade_hit_rows(x["shade_hit"])
    np.savez_compressed(HERE / "ref_shading.npz", seed=np.array([4096, 7], np.int64),
                        digest=np.array(shading_digest(x)),
                        shade=O.ref_shade_rows(x["shade"]),
                        falloff=O.ref_falloff_rows(x["falloff"][:, 0], x["falloff"][:, 1]),
                        lambert=O.ref_lambert_rows(x["lambert"]), ggx=O.ref_ggx_rows(x["ggx"]),
                        tri_data=td, tri_material=tm, shade_hit_contrib=hc, shade_hit_ray=hr, shade_hit_cast=hk)


def main() -> None:
    O.build()
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "shading":
        shading()
        print("shading fixture written to", HERE)
        return
    if not O.ref_available():
        raise SystemExit("reference harness not built: the reference sources are needed")

    # Small scene, every ray.
    s = P.generate_scene(16, 6, False, 7)
    nodes, verts, s2t = O.ref_build_sbvh(s.tri_verts)
    cam = O.ref_camera_def((0.125, -0.075, 0.15), (0.0, 0.8, -0.6), (0.0, 0.6, 0.8), math.radians(60.0), (64, 64))
    rays = O.gen_primary(cam, (64, 64))
    hits, dbg = O.ref_cast_rays(nodes, verts, rays, debug=True)
    np.savez_compressed(HERE / "ref_small.npz", nodes=nodes, slot_to_tri=s2t, verts=verts, cam=cam, hits=hits, debug=dbg,
                        scene=np.array([16, 6, 0, 7], np.int64), digest=np.array(scene_digest(s.tri_verts)))

    # Plain closest-hit configuration scene.
    g, c, rot, seed = P.STANDARD_SCENES["c1_64_100"]
    s = P.generate_scene(g, c, rot, seed)
    nodes, verts, s2t = O.ref_build_sbvh(s.tri_verts)
    cam = O.ref_camera_def(C1_CAM["pos"], C1_CAM["dir"], C1_CAM["up"], math.radians(C1_CAM["vfov"]), C1_CAM["res"])
    rays = O.gen_primary(cam, C1_CAM["res"])
    sub = rays[::16].copy()
    hits, dbg = O.ref_cast_rays(nodes, verts, sub, debug=True)
    inc = incoherent_rays(1.0, 4096, 11)
    inc_hits = O.ref_cast_rays(nodes, verts, inc)
    np.savez_compressed(HERE / "ref_c1.npz", nodes=nodes, slot_to_tri=s2t, cam=cam, hits=hits, debug=dbg,
                        inc_rays=inc, inc_hits=inc_hits, scene=np.array([g, c, int(rot), seed], np.int64),
                        digest=np.array(scene_digest(s.tri_verts)))

    # Triangle test on random pairs, including near-parallel rays and edge hits.
    rng = np.random.default_rng(5)
    n = 2000
    tris = np.zeros(n, O.TRI_VERTS_DTYPE)
    p0 = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    e1 = rng.uniform(-1, 1, (n, 3)).astype(np.float32) * rng.choice([1e-3, 0.1, 1.0], (n, 1)).astype(np.float32)
    e2 = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    tris["v0"][:, :3] = p0
    tris["v1"][:, :3] = p0 + e1
    tris["v2"][:, :3] = p0 + e2
    orig = rng.uniform(-2, 2, (n, 3)).astype(np.float32)
    target = p0 + rng.uniform(-0.2, 1.0, (n, 1)).astype(np.float32) * e1 + rng.uniform(-0.2, 1.0, (n, 1)).astype(np.float32) * e2
    dirs = (target - orig).astype(np.float32)
    out = np.zeros((n, 4), np.float32)
    ref = O.ref()
    for i in range(n):
        tuv = np.zeros(3, np.float32)
        h = ref.ref_intersect_tri(tris[i:i + 1].ctypes.data, orig[i].ctypes.data, dirs[i].ctypes.data, tuv.ctypes.data)
        out[i] = (float(h), *tuv) if h else (0.0, 0.0, 0.0, 0.0)
    np.savez_compressed(HERE / "ref_isect.npz", tris=tris, origins=orig, dirs=dirs, out=out)

    # Halton table as written in the reference.
    src = (O.REFERENCE_ROOT / "source/phantasy_engine/screens/GameScreen.cpp").read_text(errors="replace")
    block = src[src.index("HALTON_SEQ[]"):]
    block = block[:block.index("};")]
    vals = [float(x) for x in re.findall(r"([0-9]*\.[0-9]+)f", block)]
    np.save(HERE / "ref_halton.npy", np.array(vals, np.float32).reshape(-1, 2))
    shading()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
