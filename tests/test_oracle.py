"""The oracle pinned against the reference: golden fixtures produced by the reference's own code
(tests/golden/make_golden.py) and, where the reference sources are present, the live reference
harness oracle/_ref/libpheref.so. CPU only."""
import math
from pathlib import Path

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from oracle import oracle as O
from tests.helpers import C1_CAM, golden_scene, load_golden, random_rays

needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")


def test_intersect_matches_reference_fixture():
    g = load_golden("ref_isect.npz")
    tris, orig, dirs, out = g["tris"], g["origins"], g["dirs"], g["out"]
    hits = 0
    for i in range(len(tris)):
        h, t, u, v = O.intersect_tri(tris[i], orig[i], dirs[i])
        assert h == bool(out[i, 0]), i
        if h:
            hits += 1
            assert (np.float32(t), np.float32(u), np.float32(v)) == tuple(out[i, 1:]), i
    assert 200 < hits < len(tris) - 200


@pytest.mark.parametrize("fixture", ["ref_small.npz", "ref_c1.npz"])
def test_castray_matches_reference_fixture(fixture):
    """oracle castRay (reference accept rule) == the reference's castRay output, bit for bit,
    including the castDebugRay traversal counters."""
    g = load_golden(fixture)
    s, nodes, verts, s2t = golden_scene(fixture)
    if fixture == "ref_small.npz":
        assert np.array_equal(verts.view(np.uint8), g["verts"].view(np.uint8))
        rays = O.gen_primary(g["cam"], (64, 64))
    else:
        rays = O.gen_primary(g["cam"], C1_CAM["res"])[::16].copy()
    hits, dbg = O.cast_rays(nodes, verts, rays, mode=O.MODE_CPU, debug=True)
    assert np.array_equal(hits.view(np.uint8), g["hits"].view(np.uint8))
    assert np.array_equal(dbg, g["debug"])
    assert (hits["triangleIndex"] != 0xFFFFFFFF).mean() > 0.5
    if "inc_rays" in g:
        inc = O.cast_rays(nodes, verts, g["inc_rays"], mode=O.MODE_CPU)
        assert np.array_equal(inc.view(np.uint8), g["inc_hits"].view(np.uint8))


def test_camera_and_jitter_match_reference_fixture():
    g = load_golden("ref_c1.npz")
    cam = O.camera_def(C1_CAM["pos"], C1_CAM["dir"], C1_CAM["up"], math.radians(60.0), C1_CAM["res"])
    assert np.array_equal(cam, g["cam"])
    pc = P.camera_def(C1_CAM["pos"], C1_CAM["dir"], C1_CAM["up"], 60.0, C1_CAM["res"])
    assert np.array_equal(P.camera_def_array(pc), g["cam"])
    table = load_halton()
    for i in range(16):
        assert np.array_equal(O.halton_jitter(i), table[i] - np.float32(0.5))
        assert P.halton_jitter(i) == tuple(float(x) for x in table[i] - np.float32(0.5))


def load_halton():
    from tests.helpers import GOLDEN
    return np.load(GOLDEN / "ref_halton.npy")


@needs_ref
@pytest.mark.parametrize("seed", [3, 4])
def test_castray_matches_live_reference(seed):
    """Random scenes, both the reference builder's tree and the project builder's tree, coherent and
    incoherent rays: the oracle reproduces castRay bit for bit."""
    s = P.generate_scene(24, 20, seed == 4, seed)
    rn, rv, _ = O.ref_build_sbvh(s.tri_verts)
    b = P.build_sbvh(s.tri_verts)
    scale = s.scale
    rays = np.concatenate([random_rays(3000, [0, 0, 0.05], [scale, scale, 0.4 * scale], seed),
                           O.gen_primary(O.camera_def((0.5 * scale, -0.3 * scale, 0.6 * scale), (0, 0.8, -0.6),
                                                      (0, 0.6, 0.8), math.radians(60), (48, 48)), (48, 48))])
    # axis-aligned directions exercise the NaN lanes of the slab test
    ax = rays[:300].copy()
    ax["dir"] = np.array([[1, 0, 0], [0, 1, 0], [0, 0, -1]], np.float32)[np.arange(300) % 3]
    ax["origin"][:, 0] = np.round(ax["origin"][:, 0] * 64) / 64
    rays = np.concatenate([rays, ax])
    for nodes, verts in ((rn, rv), (b.nodes, b.verts)):
        mine, dbg = O.cast_rays(nodes, verts, rays, mode=O.MODE_CPU, debug=True)
        ref, rdbg = O.ref_cast_rays(nodes, verts, rays, debug=True)
        assert np.array_equal(mine.view(np.uint8), ref.view(np.uint8))
        assert np.array_equal(dbg, rdbg)


@needs_ref
def test_camera_def_matches_live_reference():
    for res in [(512, 512), (1920, 1080), (64, 48)]:
        a = O.camera_def((1, 2, 3), (0.1, 0.9, -0.3), (0, 0.3, 0.9), math.radians(47.0), res)
        b = O.ref_camera_def((1, 2, 3), (0.1, 0.9, -0.3), (0, 0.3, 0.9), math.radians(47.0), res)
        assert np.array_equal(a, b)


def test_gpu_rule_matches_cpu_rule_except_tmax():
    """The GPU accept rule (tMin <= t < tMax) gives the CPU rule's result except for hits exactly at
    tMax; on random rays they agree on every ray."""
    g = load_golden("ref_c1.npz")
    s, nodes, verts, s2t = golden_scene("ref_c1.npz")
    rays = g["inc_rays"]
    a = O.cast_rays(nodes, verts, rays, mode=O.MODE_CPU)
    b = O.cast_rays(nodes, verts, rays, mode=O.MODE_GPU)
    hit = a["triangleIndex"] != 0xFFFFFFFF
    assert np.array_equal(a["triangleIndex"], b["triangleIndex"])
    assert np.array_equal(a[hit].view(np.uint8), b[hit].view(np.uint8))
    assert np.all(b["t"][~hit] == rays["tMax"][~hit])


def test_bvh_traversal_matches_brute_force():
    s = P.generate_scene(12, 8, True, 9)
    b = P.build_sbvh(s.tri_verts)
    rays = random_rays(4000, [0, 0, 0.02], [s.scale, s.scale, 0.3 * s.scale], 21)
    tris = np.zeros(len(s.tri_verts), P.TRI_VERTS_DTYPE)
    tris["v0"][:, :3] = s.tri_verts[:, 0:3]
    tris["v1"][:, :3] = s.tri_verts[:, 3:6]
    tris["v2"][:, :3] = s.tri_verts[:, 6:9]
    bf = O.brute_closest(tris, rays, mode=O.MODE_GPU)
    bvh = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
    ident = np.arange(len(tris), dtype=np.uint32)
    # express the BVH result in original triangle ids for the comparator
    bvh_orig = bvh.copy()
    hit = bvh["triangleIndex"] != 0xFFFFFFFF
    bvh_orig["triangleIndex"][hit] = b.slot_to_tri[bvh["triangleIndex"][hit]]
    r = O.compare_closest(bvh_orig, bf, rays, ident, tris)
    assert r["ok"], r
    assert r["near_ties"] <= 4


def test_sincos_accuracy_and_pcg_reference_stream():
    xs = np.linspace(0, 1, 40001, endpoint=False, dtype=np.float32)
    err = 0.0
    for x in xs[::7]:
        s, c = O.sincos_2pi(float(x))
        err = max(err, abs(s - math.sin(2 * math.pi * float(x))), abs(c - math.cos(2 * math.pi * float(x))))
    assert err < 3e-7
    # pcg32_srandom_r(42, 54) first outputs, as printed by the PCG reference demo
    import ctypes as C
    st = (C.c_uint64 * 2)()
    L = O.lib()
    L.oracle_pcg_seed.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
    L.oracle_pcg_seed(C.addressof(st), 42, 54)
    got = [L.oracle_pcg_next(C.addressof(st)) for _ in range(6)]
    assert got == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


def test_texel_sampling_rule_and_srgb_table():
    """Nearest-texel rule of the reference's texture objects (normalized coordinates, wrap):
    floor(frac(c) * n) with n wrapping to 0; the sRGB table is powf(b / 255, 2.2) correctly rounded."""
    n = 4
    cases = {0.0: 0, 0.2499: 0, 0.25: 1, 0.999: 3, 1.0: 0, 1.3: 1, -0.25: 3, -1.0: 0, 7.75: 3,
             float("nan"): 0, float("inf"): 0, float("-inf"): 0}
    for c, want in cases.items():
        assert O.texel_coord(c, n) == want, c
    # frac of a tiny negative coordinate rounds to 1.0f: that texel wraps to 0
    assert O.texel_coord(-1e-9, 37) == 0
    for c in np.random.default_rng(5).uniform(-3, 3, 2000).astype(np.float32):
        f = np.float32(c) - np.floor(np.float32(c))
        want = int(np.float32(f) * np.float32(37))
        assert O.texel_coord(float(c), 37) == (0 if want >= 37 else want)
    t = O.srgb_table()
    assert t[0] == 0.0 and t[255] == 1.0 and np.all(np.diff(t) > 0)
    exact = (np.arange(256, dtype=np.float32) / np.float32(255)).astype(np.float64) ** np.float64(np.float32(2.2))
    assert np.array_equal(t, exact.astype(np.float32))


def test_oracle_constant_textures_equal_material_constants():
    """A texture whose every texel encodes a material's constants renders the frame of the constants:
    albedo rgb = sRGB table entry, alpha 255 -> 1, roughness 255 -> 1, metallic 0 -> 0."""
    s = P.generate_scene(24, 20, True, 7)
    b = P.build_sbvh(s.tri_verts)
    datas = s.datas.copy()
    for name in ("uv0", "uv1", "uv2"):
        datas[name] = np.random.default_rng(1).uniform(-2, 2, (len(datas), 2))
    slot_datas = b.slot_datas(datas)
    srgb = O.srgb_table()
    mats = s.materials.copy()
    mats["albedo"][:, :3] = srgb[77]
    mats["texIndex"][:] = -1
    tex = [np.full((5, 7, 4), 77, np.uint8), np.full((3, 3), 255, np.uint8), np.zeros((2, 2, 2), np.uint8)]
    tex[0][..., 3] = 255
    textured = mats.copy()
    textured["texIndex"][:] = [0, 1, 2, -1]
    textured["albedo"][:] = 0.5
    textured["roughness"] = 0.25
    textured["metallic"] = 0.75
    k = s.scale
    res = (64, 48)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
    from phantasyenginetestbed_gb300.renderer import make_lights
    lights = make_lights(np.array([(0.5, 0.5, 2.0)], np.float32) * np.float32(k), range_=1000.0 * k)
    a = O.render_frame(b.nodes, b.verts, slot_datas, mats, lights, cam, res, (0.0, 0.0), cam_pos, 3, 0)
    t = O.render_frame(b.nodes, b.verts, slot_datas, textured, lights, cam, res, (0.0, 0.0), cam_pos, 3, 0,
                       textures=tex)
    assert np.array_equal(a[0], t[0]) and np.array_equal(a[1], t[1]) and np.array_equal(a[2], t[2])
    assert a[0][..., :3].max() > 0.01


def test_oracle_scaling_pass_reproduces_linear_images():
    """Bilinear taps reproduce an affine image exactly away from the clamped border, and the four
    symmetric taps average to the value at the destination pixel's mapped centre."""
    W, H = 64, 40
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    img = np.zeros((H, W, 4), np.float32)
    img[..., 0] = 0.01 * (xx + 0.5) + 0.002 * (yy + 0.5)
    img[..., 1] = 0.5
    img[..., 2] = 0.03 * (yy + 0.5)
    for dst in ((96, 60), (32, 20), (64, 40)):
        out = O.scale(img, dst)
        dy, dx = np.mgrid[0:dst[1], 0:dst[0]].astype(np.float64)
        cx = (dx + 0.5) / dst[0] * W
        cy = (dy + 0.5) / dst[1] * H
        inner = (cx > 1.5) & (cx < W - 1.5) & (cy > 1.5) & (cy < H - 1.5)
        want_r = 0.01 * cx + 0.002 * cy
        assert np.abs(out[..., 0] - want_r)[inner].max() < 1e-5
        assert np.abs(out[..., 2] - 0.03 * cy)[inner].max() < 1e-5
        assert np.all(out[..., 1] == np.float32(0.5)) and np.all(out[..., 3] == 1.0)
    # a viewport of the lower-left 32 x 20 texels stretched over the destination: taps reach at most one
    # texel past it (clamping happens only at the texture edge, as in GL)
    out = O.scale(img, (64, 40), viewport=(32, 20))
    assert out[..., 0].max() <= img[:21, :33, 0].max() + 1e-6
    assert out[..., 0].max() > img[:20, :32, 0].max() - 0.02


def test_oracle_velocity_for_camera_motion():
    """TAA velocity restatement: 0 everywhere for an unchanged camera; a sideways camera move gives
    surface points a velocity against the move (larger for nearer points) and leaves directions at
    infinity (misses) still."""
    s = P.generate_scene(24, 20, True, 7)
    b = P.build_sbvh(s.tri_verts)
    slot_datas = b.slot_datas(s.datas)
    k = s.scale
    res = (64, 48)
    from phantasyenginetestbed_gb300.renderer import make_lights
    lights = make_lights(np.array([(0.5, 0.5, 2.0)], np.float32) * np.float32(k), range_=1000.0 * k)
    # look slightly above the horizon so that some pixels miss
    up = np.array([0.0, 0.2, 0.98]); d = np.array([0.0, 0.98, -0.2])
    pos0 = np.array([0.5 * k, -0.3 * k, 0.3 * k])
    cam0 = O.camera_def(pos0, d, up, math.radians(60), res)
    vel = np.full((res[1], res[0], 2), np.nan, np.float32)
    O.render_frame(b.nodes, b.verts, slot_datas, s.materials, lights, cam0, res, (0.1, -0.2), pos0, 3, 0,
                   prev_cam=cam0, velocity_out=vel)
    assert np.all(vel == 0.0)
    right = cam0[6:9] / np.linalg.norm(cam0[6:9])
    pos1 = pos0 + 0.02 * k * right
    cam1 = O.camera_def(pos1, d, up, math.radians(60), res)
    O.render_frame(b.nodes, b.verts, slot_datas, s.materials, lights, cam1, res, (0.0, 0.0), pos1, 3, 1,
                   prev_cam=cam0, velocity_out=vel)
    rays = O.gen_primary(cam1, res)   # row-major ray order, no jitter (as the frame above)
    h = O.cast_rays(b.nodes, b.verts, rays)
    hits = (h["triangleIndex"] != 0xFFFFFFFF).reshape(res[1], res[0])
    assert hits.any() and (~hits).any()
    assert np.all(vel[..., 0][hits] < 0) and np.all(vel[..., 1][hits] == 0.0)   # a move along the image x axis
    assert np.all(vel[~hits] == 0.0)


# --- shading, sampling and hit interpretation against the reference's own functions ----------------
# Tolerance of the shaded outputs: 1e-4 absolute per channel (linear FP32). Observed maxima on 1e5
# seeded rows (x86-64 host): shade 2.9e-6 (outputs up to 102), falloffFactor 1.2e-7, sampleLambertian
# 4.5e-7, sampleGgx 1.1e-5, shadeHit contribution 4.8e-7 and shadow-ray direction / length 8.3e-7;
# retrieveTriData bit-identical. The differences come from the oracle's integer powers as products
# (powf in CudaPbr.cuh) and its sin/cos(2 pi r) polynomial (cos/sin of a float angle in the reference).
SHADE_TOL = 1e-4
needs_ref_shading = pytest.mark.skipif(not O.ref_shading_available(), reason="reference sources not present")


def _compare_shading(x, ref, tol=SHADE_TOL):
    """Max abs error per function of the oracle against reference outputs `ref` on input rows `x`."""
    err = {}
    err["shade"] = float(np.abs(O.shade_rows(x["shade"]) - ref["shade"]).max())
    err["falloff"] = float(np.abs(O.falloff_rows(x["falloff"][:, 0], x["falloff"][:, 1]) - ref["falloff"]).max())
    err["lambert"] = float(np.abs(O.lambert_rows(x["lambert"]) - ref["lambert"]).max())
    err["ggx"] = float(np.abs(O.ggx_rows(x["ggx"]) - ref["ggx"]).max())
    d, r, h = x["tri_data"]
    td, tm = O.retrieve_tri_data(d, r, h)
    assert np.array_equal(td.view(np.uint32), ref["tri_data"].view(np.uint32)), "retrieveTriData is not bit-identical"
    assert np.array_equal(tm, ref["tri_material"])
    hc, hr, hk = O.shade_hit_rows(x["shade_hit"])
    err["shade_hit"] = float(np.abs(hc - ref["shade_hit_contrib"]).max())
    # The light casts a shadow ray when a channel exceeds 1e-4 (MaterialKernel.cu:83-85); rows whose
    # largest channel lies within the tolerance of that threshold may decide either way.
    edge = np.abs(ref["shade_hit_contrib"].max(axis=1) - np.float32(1e-4)) <= tol
    assert np.array_equal(hk[~edge], ref["shade_hit_cast"][~edge])
    both = (hk == 1) & (ref["shade_hit_cast"] == 1)
    assert np.array_equal(hr[both, 0:4], ref["shade_hit_ray"][both, 0:4])   # origin = hit position, tMin = 0.001
    err["shadow_ray"] = float(np.abs(hr[both, 4:8] - ref["shade_hit_ray"][both, 4:8]).max()) if both.any() else 0.0
    assert both.sum() > len(hk) // 10
    for k, e in err.items():
        assert e <= tol, (k, e)
    return err


def test_shading_matches_reference_fixture():
    """The oracle's shading restatement against the reference's own functions' outputs (fixture)."""
    from tests.helpers import shading_inputs
    g = load_golden("ref_shading.npz")
    n, seed = (int(v) for v in g["seed"])
    x = shading_inputs(n, seed)
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).parent / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    assert mg.shading_digest(x) == str(g["digest"]), "input rows differ from the fixture's"
    _compare_shading(x, g)


@needs_ref_shading
def test_shading_matches_live_reference_on_1e5_rows():
    """shade, falloffFactor, sampleLambertian, sampleGgx, retrieveTriData and shadeHit compiled from the
    reference's own sources, fed the same 100,000 rows (and the same uniform numbers) as the oracle."""
    from tests.helpers import shading_inputs
    x = shading_inputs(100_000, 1)
    d, r, h = x["tri_data"]
    td, tm = O.ref_retrieve_tri_data(d, r, h)
    hc, hr, hk = O.ref_shade_hit_rows(x["shade_hit"])
    ref = {"shade": O.ref_shade_rows(x["shade"]), "falloff": O.ref_falloff_rows(x["falloff"][:, 0], x["falloff"][:, 1]),
           "lambert": O.ref_lambert_rows(x["lambert"]), "ggx": O.ref_ggx_rows(x["ggx"]), "tri_data": td,
           "tri_material": tm, "shade_hit_contrib": hc, "shade_hit_ray": hr, "shade_hit_cast": hk}
    err = _compare_shading(x, ref)
    print("max abs error against the reference:", err)
