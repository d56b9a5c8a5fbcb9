"""Per-ray work figures for the roofline: castDebugRay's mean nodesVisited and triangle tests per
stage, computed by the oracle on the exact inputs of bench.py's workloads, written to
profiles/work_per_ray.json.

Algorithmic bytes per ray (used by bench.py's roofline.achieved):
  closest hit: 48 B ray I/O (32 in + 16 out) + 64 * n_node + 48 * n_tri
  any hit:     33 B ray I/O (32 in + 1 out)  + 64 * n_node + 48 * n_tri
  a shaded hit adds 64 B of TriangleData.

Frame figures are written for the tree of the reference's own builder ("reference", the tree the
frame benchmark uses) and for this project's builder ("project").

Run: python oracle/work_figures.py
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path[0] = str(ROOT)

import phantasyenginetestbed_gb300 as P  # noqa: E402
from phantasyenginetestbed_gb300.renderer import make_lights  # noqa: E402
from oracle import oracle as O  # noqa: E402

FRAME_SCENE = "c2_256_2000"
FRAME_RES = (1920, 1080)
FRAME_SEED = 2024
CAM_DIR = (0.0, 0.8, -0.6)
CAM_UP = (0.0, 0.6, 0.8)


class _Tree:
    def __init__(self, nodes, verts, s2t):
        self.nodes, self.verts, self.slot_to_tri = nodes, verts, s2t

    def slot_datas(self, datas):
        return np.ascontiguousarray(datas[self.slot_to_tri])


def frame_setup(scene_name=FRAME_SCENE, res=FRAME_RES, builder="project"):
    """builder "reference": the reference's own buildStaticFrom + sanitizeBVH (oracle/_ref); "project":
    this project's SBVH builder."""
    s = P.standard_scene(scene_name)
    b = _Tree(*O.ref_build_sbvh(s.tri_verts)) if builder == "reference" else P.build_sbvh(s.tri_verts)
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, CAM_DIR, CAM_UP, math.radians(60.0), res)
    lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
    return s, b, cam, cam_pos, lights


def frame_work(builder):
    s, b, cam, cam_pos, lights = frame_setup(builder=builder)
    work = np.zeros(8, np.uint64)
    jit = P.halton_jitter(0)
    _, _, counts = O.render_frame(b.nodes, b.verts, b.slot_datas(s.datas), s.materials, lights, cam, FRAME_RES, jit,
                                  cam_pos, FRAME_SEED, 0, work=work)
    stages = ["primary", "primary_shadow", "bounce", "bounce_shadow"]
    out = {"bvh": {"nodes": len(b.nodes), "slots": len(b.verts)}, "stages": {}}
    for i, st in enumerate(stages):
        n = int(counts[i])
        out["stages"][st] = {"rays": n, "n_node": float(work[2 * i]) / n, "n_tri": float(work[2 * i + 1]) / n}
    return out


def main() -> None:
    out = {"workload": f"wavefront frame {FRAME_SCENE} {FRAME_RES[0]}x{FRAME_RES[1]} seed {FRAME_SEED} frame 0",
           "trees": {}}
    # the tree the frame benchmark uses (the reference's own builder) and this project's builder
    for builder in ("reference", "project"):
        if builder == "reference" and not O.ref_available():
            continue
        out["trees"][builder] = frame_work(builder)
    # plain closest-hit primary rays of the 64x64-cell scene, 512x512
    s1 = P.standard_scene("c1_64_100")
    b1 = P.build_sbvh(s1.tri_verts)
    cam1 = O.camera_def((0.5, -0.3, 0.6), CAM_DIR, CAM_UP, math.radians(60.0), (512, 512))
    rays = O.gen_primary(cam1, (512, 512))
    _, dbg = O.cast_rays(b1.nodes, b1.verts, rays, debug=True)
    out["c1_primary"] = {"rays": len(rays), "n_node": float(dbg[:, 0].mean()), "n_tri": float(dbg[:, 1].mean())}
    path = ROOT / "profiles" / "work_per_ray.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(path.read_text())


if __name__ == "__main__":
    main()
