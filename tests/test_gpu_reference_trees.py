"""GPU parity on trees built by the reference's own host builder (buildStaticFrom + sanitizeBVH,
StaticBVHBuilder.cpp:213-260, compiled from the reference sources), at benchmark scale: the
155,072-triangle frame scene (256x256-cell heightfield + 2000 rotated cubes) and one scene of the
uneven-batch mix. These are the trees a drop-in caller hands the library; the other GPU tests mostly
use this project's builder, whose slot order differs.

Covered: every 1920x1080 primary ray (closest hit) and a shadow ray per hit (any hit), 400K incoherent
rays, on the binary, 4-wide and 8-wide layouts of the same tree; one full 1080p wavefront frame on the
binary and 8-wide layouts; and a batched launch over two reference-built scenes. Parity rule as everywhere: closest hits equal (or a documented near-tie), any
hits and frames (1e-4 absolute per channel) against the oracle on the same tree."""
import math

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300 import native as N
from phantasyenginetestbed_gb300.batch import ANY, CLOSEST, Batch
from phantasyenginetestbed_gb300.renderer import READ_RAW, READ_ROUGHNESS, CudaTracerRenderer, make_lights
from oracle import oracle as O
from tests.helpers import C1_CAM, cam_struct, device_empty, from_device, random_rays, ref_built_scene, to_device

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_available(), reason="reference harness not built (no reference sources)")]

RES = (1920, 1080)


def _frame_scene():
    s, t = ref_built_scene("c2_256_2000")
    assert len(s.tri_verts) == 155_072
    return s, t


def _camera(s, res):
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    return cam_pos, O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)


def _shadow_rays(rays, hits, light):
    m = hits["triangleIndex"] != 0xFFFFFFFF
    pos = rays["origin"][m] + rays["dir"][m] * hits["t"][m][:, None]
    d = np.asarray(light, np.float32) - pos
    dist = np.linalg.norm(d, axis=1)
    out = np.zeros(len(pos), P.RAY_IN_DTYPE)
    out["origin"] = pos.astype(np.float32)
    out["dir"] = (d / dist[:, None]).astype(np.float32)
    out["tMin"] = np.float32(1e-3)
    out["tMax"] = dist.astype(np.float32)
    return out


def test_reference_tree_is_accepted_with_its_wide_layout():
    """Upload validates the reference tree; every grandchild box lies inside its parent box, so the
    4-wide collapse and the 8-wide compressed layout are built for it."""
    s, t = _frame_scene()
    assert P.validate_bvh(t.nodes, len(t.verts)) <= 64
    scene = P.Scene(t.nodes, t.verts)
    layout, wide = scene.layout()
    assert layout == N.LAYOUT_BINARY and wide == 3
    scene.close()


@pytest.mark.parametrize("layout", [N.LAYOUT_BINARY, N.LAYOUT_WIDE4, N.LAYOUT_WIDE8], ids=["binary", "wide4", "wide8"])
def test_every_1080p_primary_ray_and_its_shadow_ray(layout):
    s, t = _frame_scene()
    scene = P.Scene(t.nodes, t.verts)
    scene.set_layout(layout)
    _, cam = _camera(s, RES)
    rays = O.gen_primary(cam, RES)
    d_rays = to_device(rays)
    d_hits = device_empty(len(rays), P.RAY_HIT_DTYPE)
    P.cast_closest(scene, d_rays, d_hits, len(rays))
    gpu = from_device(d_hits, P.RAY_HIT_DTYPE)
    want = O.cast_rays(t.nodes, t.verts, rays, mode=O.MODE_GPU)
    rep = O.compare_closest(gpu, want, rays, t.slot_to_tri, t.verts)
    assert rep["ok"], {k: v for k, v in rep.items() if k != "rays"}
    assert rep["hits"] > 0.3 * len(rays)
    shadow = _shadow_rays(rays, want, np.array([0.5, 0.5, 2.0], np.float32) * np.float32(s.scale))
    d_sh = to_device(shadow)
    d_vis = device_empty(len(shadow), np.uint8)
    P.cast_any(scene, d_sh, d_vis, len(shadow))
    assert np.array_equal(from_device(d_vis, np.uint8), O.any_rays(t.nodes, t.verts, shadow))
    assert scene.status() == 0
    scene.close()


@pytest.mark.parametrize("layout", [N.LAYOUT_BINARY, N.LAYOUT_WIDE4, N.LAYOUT_WIDE8], ids=["binary", "wide4", "wide8"])
def test_400k_incoherent_rays(layout):
    s, t = _frame_scene()
    scene = P.Scene(t.nodes, t.verts)
    scene.set_layout(layout)
    k = s.scale
    rays = random_rays(400_000, [0, 0, 0.02 * k], [k, k, 0.3 * k], 404, tmin=1e-3)
    d_rays = to_device(rays)
    d_hits = device_empty(len(rays), P.RAY_HIT_DTYPE)
    P.cast_closest(scene, d_rays, d_hits, len(rays))
    rep = O.compare_closest(from_device(d_hits, P.RAY_HIT_DTYPE), O.cast_rays(t.nodes, t.verts, rays, mode=O.MODE_GPU),
                            rays, t.slot_to_tri, t.verts)
    assert rep["ok"], {k: v for k, v in rep.items() if k != "rays"}
    limited = rays.copy()
    limited["tMax"] = np.float32(0.25 * k)
    d_lim = to_device(limited)
    d_vis = device_empty(len(rays), np.uint8)
    P.cast_any(scene, d_lim, d_vis, len(rays))
    assert np.array_equal(from_device(d_vis, np.uint8), O.any_rays(t.nodes, t.verts, limited))
    scene.close()


@pytest.mark.parametrize("layout", [N.LAYOUT_BINARY, N.LAYOUT_WIDE8], ids=["binary", "wide8"])
def test_1080p_frame_on_the_reference_tree(layout):
    s, t = _frame_scene()
    datas = t.slot_datas(s.datas)
    scene = P.Scene(t.nodes, t.verts, datas, s.materials)
    scene.set_layout(layout)
    cam_pos, cam = _camera(s, RES)
    lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(s.scale), range_=1000.0 * s.scale)
    r = CudaTracerRenderer(use_graph=True)
    r.setStaticScene(scene)
    r.setTargetResolution(RES)
    r.set_seed(2024, 3)
    r.resetTAA()
    jit = P.halton_jitter(3)
    r.set_camera_def(cam_struct(cam), cam_pos, jit)
    r.render(lights)
    raw = r.read(READ_RAW)
    rough = r.read(READ_ROUGHNESS)
    counts = r.ray_counts()
    ref, ref_rough, ref_counts = O.render_frame(t.nodes, t.verts, datas, s.materials, lights, cam, RES, jit, cam_pos,
                                                2024, 3)
    d = np.abs(raw.astype(np.float64) - ref.astype(np.float64))
    bad = (d > 1e-4).any(axis=-1)
    assert bad.mean() <= 1e-5, f"{bad.sum()} pixels off by more than 1e-4 (max {d.max()})"
    assert np.array_equal(rough, ref_rough)
    assert np.array_equal(counts, ref_counts.astype(np.uint64))
    assert scene.status() == 0
    r.close()
    scene.close()


def test_batch_over_reference_trees():
    """One batched launch over the 10K and 155K scenes of the uneven-batch mix, both reference-built."""
    import torch
    built = [ref_built_scene("c3_10k"), ref_built_scene("c3_155k")]
    scenes = [P.Scene(t.nodes, t.verts) for _, t in built]
    rng = np.random.default_rng(31)
    items, host = [], []
    for i, n in enumerate([70_000, 3_000, 250_000, 1_024, 40_000, 120_000]):
        si = i % 2
        s = built[si][0]
        k = s.scale
        rays = random_rays(n, [0, 0, 0.02 * k], [k, k, 0.3 * k], 900 + i, tmin=1e-3)
        kind = CLOSEST if rng.random() < 0.7 else ANY
        if kind == ANY:
            rays["tMax"] = np.float32(0.3 * k)
        items.append((si, kind, n, to_device(rays), device_empty(n, P.RAY_HIT_DTYPE if kind == CLOSEST else np.uint8)))
        host.append(rays)
    b = Batch(scenes, items, use_graph=True)
    b.launch()
    torch.cuda.synchronize()
    for (si, kind, n, _, d_out), rays in zip(items, host):
        t = built[si][1]
        if kind == CLOSEST:
            rep = O.compare_closest(from_device(d_out, P.RAY_HIT_DTYPE), O.cast_rays(t.nodes, t.verts, rays, mode=O.MODE_GPU),
                                    rays, t.slot_to_tri, t.verts)
            assert rep["ok"], {k: v for k, v in rep.items() if k != "rays"}
        else:
            assert np.array_equal(from_device(d_out, np.uint8), O.any_rays(t.nodes, t.verts, rays))
    for sc in scenes:
        assert sc.status() == 0
    b.close()
