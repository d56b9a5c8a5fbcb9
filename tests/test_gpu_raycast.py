"""GPU parity of the ray-cast kernels against the oracle and the reference's golden fixtures.

Rule (closest hit): hit/miss identical, the original triangle identical with t/u/v within 1e-5
relative (bit-exact in practice), or a documented near-tie (|dt|/t <= 1e-6, confirmed by the oracle's
triangle test). Any hit: identical, bit for bit.
"""
import math

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from oracle import oracle as O
from tests.helpers import (C1_CAM, built_scene, cam_struct, device_empty, from_device, golden_scene, load_golden,
                           random_rays, to_device)

pytestmark = pytest.mark.gpu

NEAR_TIE_BUDGET = 1e-4  # fraction of rays allowed to be documented near-ties


def _gpu_closest(scene, rays, kind="persistent"):
    import torch
    d_rays = to_device(rays)
    d_hits = device_empty(len(rays), P.RAY_HIT_DTYPE)
    fn = P.cast_closest if kind == "persistent" else P.cast_closest_plain
    fn(scene, d_rays, d_hits, len(rays))
    torch.cuda.synchronize()
    return from_device(d_hits, P.RAY_HIT_DTYPE)


def _gpu_any(scene, rays):
    import torch
    d_rays = to_device(rays)
    d_out = device_empty(len(rays), np.uint8)
    P.cast_any(scene, d_rays, d_out, len(rays))
    torch.cuda.synchronize()
    return from_device(d_out, np.uint8)


def _check(report, n):
    assert report["ok"], {k: (v[:20] if isinstance(v, list) else v) for k, v in report.items()}
    assert report["near_ties"] <= max(2, NEAR_TIE_BUDGET * n), report["near_ties"]


@pytest.mark.parametrize("kind", ["persistent", "plain"])
def test_closest_matches_reference_fixture_c1(kind):
    """The reference's own castRay output over the reference builder's SBVH (fixture), every 16th of
    the 512x512 primary rays plus 4096 incoherent rays."""
    g = load_golden("ref_c1.npz")
    s, nodes, verts, s2t = golden_scene("ref_c1.npz")
    scene = P.Scene(nodes, verts)
    rays = O.gen_primary(g["cam"], C1_CAM["res"])[::16].copy()
    gpu = _gpu_closest(scene, rays, kind)
    ref = g["hits"].copy()
    miss = ref["triangleIndex"] == 0xFFFFFFFF
    ref["t"][miss] = rays["tMax"][miss]   # the GPU miss convention (t = tMax, u = v = 0)
    ref["u"][miss] = 0
    ref["v"][miss] = 0
    _check(O.compare_closest(gpu, ref, rays, s2t, verts), len(rays))
    inc = g["inc_rays"]
    gpu = _gpu_closest(scene, inc, kind)
    ref = g["inc_hits"].copy()
    miss = ref["triangleIndex"] == 0xFFFFFFFF
    ref["t"][miss] = inc["tMax"][miss]
    ref["u"][miss] = 0
    ref["v"][miss] = 0
    _check(O.compare_closest(gpu, ref, inc, s2t, verts), len(inc))


def test_small_fixture_every_ray_and_primary_generation():
    g = load_golden("ref_small.npz")
    s, nodes, verts, s2t = golden_scene("ref_small.npz")
    scene = P.Scene(nodes, verts)
    import torch
    for order in (0, 1):
        d_rays = device_empty(64 * 64, P.RAY_IN_DTYPE)
        P.gen_primary_rays(d_rays, cam_struct(g["cam"]), (64, 64), order=order)
        torch.cuda.synchronize()
        gpu_rays = from_device(d_rays, P.RAY_IN_DTYPE)
        want = O.gen_primary(g["cam"], (64, 64), order=order)
        assert np.array_equal(gpu_rays.view(np.uint8), want.view(np.uint8))
    rays = O.gen_primary(g["cam"], (64, 64))
    gpu = _gpu_closest(scene, rays)
    orc = O.cast_rays(nodes, verts, rays, mode=O.MODE_GPU)
    _check(O.compare_closest(gpu, orc, rays, s2t, verts), len(rays))


@pytest.mark.parametrize("name", ["c1_64_100", "c2_256_2000"])
def test_closest_and_any_full_size_vs_oracle(name):
    """Every primary ray of the configuration (512x512 for the plain scene, 1920x1080 for the
    wavefront scene), incoherent bounce-like rays, and shadow rays, over the project builder's SBVH."""
    s, b = built_scene(name)
    scene = P.Scene(b.nodes, b.verts)
    if name == "c1_64_100":
        cam = O.camera_def(C1_CAM["pos"], C1_CAM["dir"], C1_CAM["up"], math.radians(60), (512, 512))
        res = (512, 512)
    else:
        k = s.scale
        cam = O.camera_def((0.5 * k, -0.3 * k, 0.6 * k), C1_CAM["dir"], C1_CAM["up"], math.radians(60), (1920, 1080))
        res = (1920, 1080)
    rays = O.gen_primary(cam, res, jitter=(0.25, -0.125))
    gpu = _gpu_closest(scene, rays)
    orc = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
    _check(O.compare_closest(gpu, orc, rays, b.slot_to_tri, b.verts), len(rays))
    assert np.array_equal(gpu["triangleIndex"] == 0xFFFFFFFF, orc["triangleIndex"] == 0xFFFFFFFF)

    # incoherent rays from the hit points
    hit = orc["triangleIndex"] != 0xFFFFFFFF
    pos = rays["origin"][hit] + rays["dir"][hit] * orc["t"][hit][:, None]
    rng = np.random.default_rng(5)
    d = rng.normal(size=pos.shape).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:, 2] = np.abs(d[:, 2])
    inc = np.zeros(len(pos), P.RAY_IN_DTYPE)
    inc["origin"] = pos.astype(np.float32)
    inc["dir"] = d.astype(np.float32)
    inc["tMin"] = np.float32(1e-3)
    inc["tMax"] = np.float32(3.4028235e38)
    inc = inc[: 400_000]
    gpu = _gpu_closest(scene, inc)
    orc2 = O.cast_rays(b.nodes, b.verts, inc, mode=O.MODE_GPU)
    _check(O.compare_closest(gpu, orc2, inc, b.slot_to_tri, b.verts), len(inc))

    # shadow rays toward a point light: any hit must be bit-identical
    light = np.array([0.5, 0.5, 2.0], np.float32) * np.float32(s.scale)
    sh = np.zeros(len(pos), P.RAY_IN_DTYPE)
    diff = (light[None, :] - pos).astype(np.float32)
    dist = np.sqrt((diff * diff).sum(1)).astype(np.float32)
    sh["origin"] = pos.astype(np.float32)
    sh["dir"] = (diff / dist[:, None]).astype(np.float32)
    sh["tMin"] = np.float32(1e-3)
    sh["tMax"] = dist
    gpu_any = _gpu_any(scene, sh)
    orc_any = O.any_rays(b.nodes, b.verts, sh)
    assert np.array_equal(gpu_any, orc_any)
    assert 0.05 < orc_any.mean() < 0.999
    assert scene.status() == 0          # no stack overflow; in the checked build, no index out of range


def test_edge_cases():
    """Axis-aligned rays on cell planes (NaN slab lanes), rays with tMin > tMax, tMax = 0, origins
    exactly on vertices, zero-length directions and NaN rays: GPU equals the oracle bit for bit."""
    s, b = built_scene("c1_64_100")
    scene = P.Scene(b.nodes, b.verts)
    rng = np.random.default_rng(3)
    n = 6000
    rays = random_rays(n, [0, 0, 0.02], [1, 1, 0.3], 17)
    k = np.arange(n)
    axes = np.array([[1, 0, 0], [0, 1, 0], [0, 0, -1], [-1, 0, 0], [0, -1, 0], [0, 0, 1]], np.float32)
    sel = k % 4 == 0
    rays["dir"][sel] = axes[(k[sel] // 4) % 6]
    rays["origin"][sel, 0] = (np.round(rays["origin"][sel, 0] * 64) / 64).astype(np.float32)
    rays["origin"][sel, 1] = (np.round(rays["origin"][sel, 1] * 64) / 64).astype(np.float32)
    rays["tMin"][k % 13 == 1] = np.float32(5.0)       # tMin > tMax for some below
    rays["tMax"][k % 13 == 1] = np.float32(1.0)
    rays["tMax"][k % 13 == 2] = np.float32(0.0)
    rays["tMax"][k % 13 == 3] = np.float32(0.05)
    tv = s.tri_verts[b.slot_to_tri[rng.integers(0, len(b.slot_to_tri), n)]]
    on_vertex = k % 13 == 4
    rays["origin"][on_vertex] = tv[on_vertex, 0:3] + np.float32(0.0)
    rays["dir"][k % 97 == 5] = 0.0
    rays["dir"][k % 89 == 6] = np.nan
    gpu = _gpu_closest(scene, rays)
    gpu_plain = _gpu_closest(scene, rays, "plain")
    orc = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
    for res in (gpu, gpu_plain):
        _check(O.compare_closest(res, orc, rays, b.slot_to_tri, b.verts), n)
    assert np.array_equal(_gpu_any(scene, rays), O.any_rays(b.nodes, b.verts, rays))


def test_sizes_zero_one_and_ragged():
    import torch
    s, b = built_scene("c1_64_100")
    scene = P.Scene(b.nodes, b.verts)
    d_rays = device_empty(1, P.RAY_IN_DTYPE)
    d_hits = device_empty(1, P.RAY_HIT_DTYPE)
    P.cast_closest(scene, d_rays, d_hits, 0)
    P.cast_any(scene, d_rays, device_empty(1, np.uint8), 0)
    for n in (1, 31, 33, 1000, 4097):
        rays = random_rays(n, [0, 0, 0.05], [1, 1, 0.4], n)
        orc = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
        for kind in ("persistent", "plain"):
            gpu = _gpu_closest(scene, rays, kind)
            _check(O.compare_closest(gpu, orc, rays, b.slot_to_tri, b.verts), n)
    torch.cuda.synchronize()


def test_invalid_scene_and_arguments_are_rejected():
    s, b = built_scene("c1_64_100")
    bad = b.nodes.copy()
    bad["iData"][0, 0] = len(bad) + 5          # child index out of range
    bad["iData"][0, 2] = 0
    with pytest.raises(P.PheError) as e:
        P.Scene(bad, b.verts)
    assert e.value.status == 2
    cyc = b.nodes.copy()
    inner = np.nonzero(cyc["iData"][:, 2] == 0)[0]
    cyc["iData"][inner[1], 0] = 0               # points back at the root
    cyc["iData"][inner[1], 2] = 0
    with pytest.raises(P.PheError):
        P.Scene(cyc, b.verts)
    scene = P.Scene(b.nodes, b.verts)
    with pytest.raises(P.PheError):
        P.cast_closest(scene, None, device_empty(4, P.RAY_HIT_DTYPE), 4)


@pytest.mark.parametrize("T", [1, 2, 3, 5, 8, 13, 32, 64])
def test_small_scenes_every_ray_vs_brute_force(T):
    """Exhaustive small cases: 1..64 random triangles (some sharing edges, some degenerate), 4096 rays
    from all around; GPU closest hit vs brute force over the triangles, GPU any hit vs the oracle."""
    rng = np.random.default_rng(T)
    tv = rng.uniform(0, 1, (T, 9)).astype(np.float32)
    if T >= 3:
        tv[1, 0:3], tv[1, 3:6] = tv[0, 0:3], tv[0, 6:9]     # shared edge
        tv[2, 6:9] = tv[2, 0:3]                               # degenerate (zero area)
    b = P.build_sbvh(tv)
    scene = P.Scene(b.nodes, b.verts)
    rays = random_rays(4096, [-0.5, -0.5, -0.5], [1.5, 1.5, 1.5], 100 + T)
    aim = rng.uniform(0.2, 0.8, (4096, 3)).astype(np.float32)
    d = aim - rays["origin"]
    rays["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tris = np.zeros(T, P.TRI_VERTS_DTYPE)
    tris["v0"][:, :3], tris["v1"][:, :3], tris["v2"][:, :3] = tv[:, 0:3], tv[:, 3:6], tv[:, 6:9]
    bf = O.brute_closest(tris, rays, mode=O.MODE_GPU)
    gpu = _gpu_closest(scene, rays)
    gpu_orig = gpu.copy()
    hit = gpu["triangleIndex"] != 0xFFFFFFFF
    gpu_orig["triangleIndex"][hit] = b.slot_to_tri[gpu["triangleIndex"][hit]]
    rep = O.compare_closest(gpu_orig, bf, rays, np.arange(T, dtype=np.uint32), tris)
    _check(rep, len(rays))
    assert hit.mean() > 0.05
    assert np.array_equal(_gpu_any(scene, rays), O.any_rays(b.nodes, b.verts, rays))


@pytest.mark.parametrize("layout", [1, 2], ids=["wide4", "wide8"])
def test_wide_layout_gives_the_binary_results(layout):
    """The 4-wide and the 8-wide compressed node layouts reach the leaves the binary layout reaches:
    closest hits (same slots except documented near-ties) and any hits identical, on coherent,
    incoherent and axis-aligned rays."""
    s, b = built_scene("c2_256_2000")
    scene = P.Scene(b.nodes, b.verts)
    lay, avail = scene.layout()
    assert lay == 0 and avail == 3
    k = s.scale
    cam = O.camera_def((0.5 * k, -0.3 * k, 0.6 * k), C1_CAM["dir"], C1_CAM["up"], math.radians(60), (640, 360))
    rays = np.concatenate([O.gen_primary(cam, (640, 360)), random_rays(100000, [0, 0, 0.02], [k, k, 0.3 * k], 9)])
    axes = np.array([[1, 0, 0], [0, 1, 0], [0, 0, -1]], np.float32)
    rays["dir"][::7] = axes[np.arange(len(rays[::7])) % 3]
    binary = _gpu_closest(scene, rays)
    binary_any = _gpu_any(scene, rays)
    scene.set_layout(layout)
    assert scene.layout() == (layout, 3)
    for kind in ("persistent", "plain"):
        wide = _gpu_closest(scene, rays, kind)
        _check(O.compare_closest(wide, binary, rays, b.slot_to_tri, b.verts), len(rays))
    assert np.array_equal(_gpu_any(scene, rays), binary_any)
    orc = O.cast_rays(b.nodes, b.verts, rays)
    _check(O.compare_closest(_gpu_closest(scene, rays), orc, rays, b.slot_to_tri, b.verts), len(rays))


def test_inverted_child_box_keeps_the_binary_layout():
    """A child box stored with lo > hi on one axis is valid input (the reference's min/max slab test
    treats it as the swapped interval) but breaks the box nesting the 4-wide collapse relies on: the
    scene offers the binary layout only, refuses the wide ones, and its casts match the oracle."""
    s, b = built_scene("c1_64_100")
    nodes = b.nodes.copy()
    root = nodes[0]
    inner = [int(root["iData"][c]) for c in range(2) if root["iData"][2 + c] == 0]
    assert inner, "root has no inner child"
    child = inner[0]
    box = nodes[child]["fData"]
    box[0], box[3] = box[3], box[0]          # first child box of that node: swap lo.x and hi.x
    assert box[0] > box[3]
    scene = P.Scene(nodes, b.verts)
    assert scene.layout() == (0, 0)
    for layout in (1, 2):
        with pytest.raises(P.PheError):
            scene.set_layout(layout)
    k = s.scale
    cam = O.camera_def((0.5 * k, -0.3 * k, 0.6 * k), C1_CAM["dir"], C1_CAM["up"], math.radians(60), (256, 256))
    rays = np.concatenate([O.gen_primary(cam, (256, 256)), random_rays(20000, [0, 0, 0.02], [k, k, 0.3 * k], 4)])
    orc = O.cast_rays(nodes, b.verts, rays)
    _check(O.compare_closest(_gpu_closest(scene, rays), orc, rays, b.slot_to_tri, b.verts), len(rays))
    assert np.array_equal(_gpu_any(scene, rays), O.any_rays(nodes, b.verts, rays))


@pytest.mark.parametrize("a", [3.16e-3, 3.17e-3, 3.2e-3, 3.25e-3, 1.0e-2])
def test_triangle_test_decision_boundaries(a):
    """One small right triangle (legs a, so det = a^2 |d.z| for a ray along d) hit by rays whose
    |det| falls on both sides of the reference's 1e-5 epsilon, aimed at points of the barycentric grid
    that include the edges u = 0, v = 0, u + v = 1 and the vertices, each also nudged by one ulp. Every
    hit/miss decision and every t, u, v bit equals the oracle's (the reference traversal restated, GPU
    accept rule), for closest and any hit. The edges lie on faces of the triangle's flat bounding box,
    so rays aimed at them also exercise the rounded slab test there. At a = 3.16e-3, a^2 < 1e-5: every
    ray misses."""
    p0 = np.array([0.25, 0.5, 0.1], np.float32)
    tv = np.concatenate([p0, p0 + np.float32([a, 0, 0]), p0 + np.float32([0, a, 0])]).astype(np.float32)[None, :]
    b = P.build_sbvh(tv)
    scene = P.Scene(b.nodes, b.verts)
    g = np.array([0.0, 0.25, 0.5, 0.75, 1.0], np.float32)
    uv = np.array([(u, v) for u in g for v in g if u + v <= 1.0], np.float32)
    aim = p0 + uv[:, :1] * np.float32(a) * np.float32([1, 0, 0]) + uv[:, 1:] * np.float32(a) * np.float32([0, 1, 0])
    aim = aim.astype(np.float32)
    aim = np.concatenate([aim, np.nextafter(aim, np.float32(-1)), np.nextafter(aim, np.float32(2))])
    dz = np.linspace(-1.0, -0.9, 64, dtype=np.float32)              # |d.z| from 1 down to 0.9
    az = np.linspace(0, 2 * np.pi, 7, endpoint=False)
    rays = []
    for z in dz:
        for phi in az:
            sxy = np.sqrt(1 - z * z)
            d = np.array([sxy * np.cos(phi), sxy * np.sin(phi), z], np.float32)
            o = (aim - d * np.float32(0.3)).astype(np.float32)
            r = np.zeros(len(aim), P.RAY_IN_DTYPE)
            r["origin"], r["dir"], r["tMin"], r["tMax"] = o, d, np.float32(1e-4), np.float32(3.4028235e38)
            rays.append(r)
    rays = np.concatenate(rays)
    bf = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
    gpu = _gpu_closest(scene, rays)
    hit = gpu["triangleIndex"] != 0xFFFFFFFF
    assert np.array_equal(hit, bf["triangleIndex"] != 0xFFFFFFFF)
    if a * a < 1e-5:
        assert not hit.any()                                         # every |det| is below the epsilon
    else:
        assert 0.02 < hit.mean() < 0.95, hit.mean()                  # both sides of the epsilon and the edges
    for f in ("t", "u", "v"):
        assert np.array_equal(gpu[f][hit].view(np.uint32), bf[f][hit].view(np.uint32)), f
    assert np.array_equal(_gpu_any(scene, rays), (bf["triangleIndex"] == 0xFFFFFFFF).astype(np.uint8))
