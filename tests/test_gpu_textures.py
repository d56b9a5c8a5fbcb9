"""Textured materials (the reference's Material with albedo / roughness / metallic texture indices,
InterpretRayHitKernel.cu:60-121, sampled like CudaBindlessTexture.cpp:66-72): the GPU frame equals the
oracle frame on a scene whose materials mix constants and textures of 1, 2 and 4 bytes per pixel,
including alpha below 0.5 (the pass-through bounce); replacing materials between frames of a replayed
graph takes effect; invalid materials and textures are refused."""
import math

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300.renderer import READ_RAW, READ_ROUGHNESS, CudaTracerRenderer, make_lights
from oracle import oracle as O
from tests.helpers import C1_CAM, cam_struct

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _textured_scene(seed=11):
    s = P.generate_scene(96, 300, True, seed)
    datas = s.datas.copy()
    # planar uv from world xy (several texture repeats, negative and > 1 coordinates included)
    k = 5.0 / s.scale
    for c, name in enumerate(["uv0", "uv1", "uv2"]):
        datas[name][:, 0] = s.tri_verts[:, 3 * c] * k - 1.3
        datas[name][:, 1] = s.tri_verts[:, 3 * c + 1] * k - 0.7
    rng = np.random.default_rng(seed)
    textures = [rng.integers(0, 256, (23, 37, 4), dtype=np.uint8),      # albedo, odd sizes
                rng.integers(0, 256, (16, 16), dtype=np.uint8),          # roughness, 1 byte per pixel
                rng.integers(0, 256, (8, 8, 2), dtype=np.uint8),         # metallic, 2 bytes per pixel
                rng.integers(0, 256, (64, 1, 4), dtype=np.uint8)]        # albedo, one column
    mats = s.materials.copy()
    choice = rng.integers(0, 6, len(mats))
    mats["texIndex"][:] = -1
    mats["texIndex"][choice == 1, 0] = 0
    mats["texIndex"][choice == 2, 1] = 1
    mats["texIndex"][choice == 3, 2] = 2
    mats["texIndex"][choice == 4] = [3, 1, 2, -1]
    mats["texIndex"][choice == 5] = [0, 1, -1, -1]
    mats["roughness"][choice == 0] = 0.35    # a specular lobe on some untextured materials
    return s, datas, mats, textures


def _render(r, cam, cam_pos, lights, frames=1):
    for f in range(frames):
        r.set_camera_def(cam_struct(cam), cam_pos, P.halton_jitter(f))
        r.render(lights)
    return r.read(READ_RAW), r.read(READ_ROUGHNESS), r.ray_counts()


def _oracle(b, slot_datas, mats, lights, cam, res, cam_pos, textures, frame=0):
    return O.render_frame(b.nodes, b.verts, slot_datas, mats, lights, cam, res, P.halton_jitter(frame), cam_pos,
                          21, frame, textures=textures)


def _compare(gpu, ref, what):
    d = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    bad = (d > TOL).any(axis=-1) if d.ndim == 3 else d > TOL
    assert bad.mean() <= 1e-5, f"{what}: {bad.sum()} pixels off by more than {TOL} (max {d.max()})"


@pytest.mark.parametrize("graph", [False, True])
def test_textured_frame_matches_oracle(graph):
    s, datas, mats, textures = _textured_scene()
    b = P.build_sbvh(s.tri_verts)
    slot_datas = b.slot_datas(datas)
    scene = P.Scene(b.nodes, b.verts, slot_datas, s.materials)
    scene.setMaterialsAndTextures(mats, textures)
    k = s.scale
    res = (320, 200)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
    lights = make_lights(np.array([(0.5, 0.5, 2.0), (0.2, 0.8, 0.9)], np.float32) * np.float32(k), range_=1000.0 * k)
    r = CudaTracerRenderer(use_graph=graph)
    r.setStaticScene(scene)
    r.setTargetResolution(res)
    r.set_seed(21, 0)
    r.resetTAA()
    raw, rough, counts = _render(r, cam, cam_pos, lights)
    ref, ref_rough, ref_counts = _oracle(b, slot_datas, mats, lights, cam, res, cam_pos, textures)
    _compare(raw, ref, "textured frame")
    assert np.array_equal(rough, ref_rough)
    assert np.array_equal(counts, ref_counts.astype(np.uint64))
    # textures actually reached the image: roughness takes values of the 1-byte texture
    assert len(np.unique(rough)) > 50

    # Replace the materials (constants only) between frames: the replayed graph must pick them up.
    plain = s.materials.copy()
    scene.setMaterialsAndTextures(plain)
    r.set_seed(21, 0)
    r.resetTAA()
    raw2, rough2, counts2 = _render(r, cam, cam_pos, lights)
    ref2, ref_rough2, ref_counts2 = _oracle(b, slot_datas, plain, lights, cam, res, cam_pos, ())
    _compare(raw2, ref2, "frame after material replacement")
    assert np.array_equal(rough2, ref_rough2)
    assert np.array_equal(counts2, ref_counts2.astype(np.uint64))
    assert not np.array_equal(raw2, raw)


def test_invalid_materials_and_textures_are_refused():
    s, datas, mats, textures = _textured_scene(12)
    b = P.build_sbvh(s.tri_verts)
    scene = P.Scene(b.nodes, b.verts, b.slot_datas(datas), s.materials)
    bad = mats.copy()
    bad["texIndex"][0, 0] = len(textures)                       # index out of range
    with pytest.raises(P.PheError):
        scene.setMaterialsAndTextures(bad, textures)
    bad = mats.copy()
    bad["texIndex"][0] = [1, -1, -1, -1]                         # albedo from a 1-byte texture
    with pytest.raises(P.PheError):
        scene.setMaterialsAndTextures(bad, textures)
    bad = mats.copy()
    bad["texIndex"][0, 2] = -2
    with pytest.raises(P.PheError):
        scene.setMaterialsAndTextures(bad, textures)
    with pytest.raises(P.PheError):                              # fewer materials than materialIndex needs
        scene.setMaterialsAndTextures(mats[:10], textures)
    with pytest.raises(P.PheError):                              # 3 bytes per pixel
        scene.setMaterialsAndTextures(s.materials, [np.zeros((4, 4, 3), np.uint8)])
    scene.setMaterialsAndTextures(mats, textures)                # the valid set still loads
    assert scene.device_bytes() > 0


def test_renderer_level_materials_call_order():
    """The reference's order (GameScreen.cpp:86-87): setMaterialsAndTextures, then setStaticScene."""
    s, datas, mats, textures = _textured_scene(13)
    b = P.build_sbvh(s.tri_verts)
    slot_datas = b.slot_datas(datas)
    scene = P.Scene(b.nodes, b.verts, slot_datas)          # no materials yet
    k = s.scale
    res = (96, 64)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
    lights = make_lights(np.array([(0.5, 0.5, 2.0)], np.float32) * np.float32(k), range_=1000.0 * k)
    r = CudaTracerRenderer()
    r.setMaterialsAndTextures(mats, textures)
    r.setStaticScene(scene)
    r.setTargetResolution(res)
    r.set_seed(21, 0)
    r.resetTAA()
    raw, rough, counts = _render(r, cam, cam_pos, lights)
    ref, ref_rough, ref_counts = _oracle(b, slot_datas, mats, lights, cam, res, cam_pos, textures)
    _compare(raw, ref, "renderer-level materials")
    assert np.array_equal(rough, ref_rough)
