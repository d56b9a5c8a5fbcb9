"""The 8-wide compressed layout on the CPU: the structure phe_bvh_wide8_build returns (every leaf of the
binary tree once, every quantized child box containing the exact boxes beneath it, exact decoding of
the grid bytes) and a scalar emulation of its traversal arithmetic (tests/cpp/wide8_emul.c) that gives
the oracle's results on reference-built and project-built trees."""
import ctypes as C
import math
import subprocess
from functools import lru_cache
from pathlib import Path

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from oracle import oracle as O
from tests.helpers import built_scene, hemisphere_rays_from_hits, random_rays

HERE = Path(__file__).resolve().parent


@lru_cache(maxsize=None)
def emul():
    so = HERE / "cpp" / "_build" / "wide8_emul.so"
    src = HERE / "cpp" / "wide8_emul.c"
    if not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
        so.parent.mkdir(exist_ok=True)
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", str(so), str(src),
                        "-lm"], check=True)
    L = C.CDLL(str(so))
    V = C.c_void_p
    L.wide8_cast.argtypes = [V, V, V, V, C.c_uint32, C.c_int, V, V, V]
    return L


def emul_cast(w, lv, verts, rays, mode):
    n = len(rays)
    hits = np.empty(n, O.RAY_HIT_DTYPE)
    vis = np.empty(n, np.uint8)
    st = np.empty((n, 3), np.uint32)
    ov = emul().wide8_cast(w.ctypes.data, lv.ctypes.data, verts.ctypes.data, rays.ctypes.data, n, mode, hits.ctypes.data,
                           vis.ctypes.data, st.ctypes.data)
    assert ov == 0
    return hits, vis, st


def decode(w):
    """Child boxes (N, 8, 6) as float64 from the node words, and the per-node masks."""
    meta = w[:, 3]
    e = np.stack([(meta >> (8 * i)) & 0xFF for i in range(3)], 1).astype(np.int64) - 128
    pp = w[:, 0:3].view(np.float32).astype(np.float64)
    b = w[:, 8:20].view(np.uint8).reshape(len(w), 3, 2, 8).astype(np.float64)  # axis, lo/hi, slot
    scale = np.ldexp(1.0, e)[:, :, None, None]
    vals = (np.float64(2 ** 23) + b) * scale + pp[:, :, None, None]
    lo = vals[:, :, 0, :].transpose(0, 2, 1)
    hi = vals[:, :, 1, :].transpose(0, 2, 1)
    return lo, hi, (meta >> 24) & 0xFF, w[:, 6] & 0xFF


def check_structure(nodes, nslots):
    w, lv, depth = P.wide8_build(nodes, nslots)
    assert 1 <= depth <= 64
    lo, hi, imask, valid = decode(w)
    # decoded bounds are exact floats on each node's grid (the kernel's fma decode is exact)
    assert np.array_equal(lo[valid[:, None] & (1 << np.arange(8)) != 0].astype(np.float32).astype(np.float64),
                          lo[valid[:, None] & (1 << np.arange(8)) != 0])
    # leaves: every binary leaf range exactly once, exact boxes inside their quantized boxes
    first = lv[:, 3]
    count = lv[:, 7]
    assert (count > 0).all()
    order = np.argsort(first)
    assert first[order][0] == 0 or True
    covered = np.zeros(nslots, np.int32)
    for f, c in zip(first, count):
        covered[f:f + c] += 1
    idx = nodes["iData"]
    bin_leaf = np.zeros(nslots, np.int32)
    for ch in (0, 1):
        leaf = idx[:, 2 + ch] > 0
        raw = idx[leaf, ch]
        for f, c in zip(np.where(raw < 0, ~raw, raw), idx[leaf, 2 + ch]):
            bin_leaf[f:f + c] += 1
    assert np.array_equal(covered, bin_leaf)
    exact = lv.view(np.float32)
    seen_nodes = np.zeros(len(w), np.int32)
    seen_nodes[0] = 1
    for n in range(len(w)):
        inner_rank = leaf_rank = 0
        for s in range(8):
            if not (valid[n] >> s) & 1:
                continue
            qlo, qhi = lo[n, s], hi[n, s]
            if (imask[n] >> s) & 1:
                c = w[n, 4] + inner_rank
                inner_rank += 1
                seen_nodes[c] += 1
                clo, chi, cval = lo[c], hi[c], valid[c]
                m = (cval & (1 << np.arange(8))) != 0
                # the child node's own children all lie inside this quantized box
                assert (clo[m] >= qlo - 0).all() and (chi[m] <= qhi + 0).all(), (n, s)
            else:
                r = w[n, 5] + leaf_rank
                leaf_rank += 1
                assert (exact[r, 0:3] >= qlo).all() and (exact[r, 4:7] <= qhi).all(), (n, s)
    assert (seen_nodes == 1).all()
    return w, lv


@pytest.mark.parametrize("name", ["c1_64_100", "c2_256_2000"])
def test_wide8_structure_project_trees(name):
    s, b = built_scene(name)
    check_structure(b.nodes, len(b.verts))


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
def test_wide8_structure_and_emulated_traversal_on_the_reference_tree():
    from tests.helpers import ref_built_scene
    s, t = ref_built_scene("c2_256_2000")
    w, lv = check_structure(t.nodes, len(t.verts))
    k = s.scale
    cam = O.camera_def((0.5 * k, -0.3 * k, 0.6 * k), (0.0, 0.8, -0.6), (0.0, 0.6, 0.8), math.radians(60), (960, 540))
    rays = O.gen_primary(cam, (960, 540))[::3].copy()
    hits, _, st = emul_cast(w, lv, t.verts, rays, 0)
    want = O.cast_rays(t.nodes, t.verts, rays, mode=O.MODE_GPU)
    rep = O.compare_closest(hits, want, rays, t.slot_to_tri, t.verts)
    assert rep["ok"], {k_: v for k_, v in rep.items() if k_ != "rays"}

    def normals(slots):
        tv = t.verts[slots]
        n = np.cross(tv["v1"][:, :3] - tv["v0"][:, :3], tv["v2"][:, :3] - tv["v0"][:, :3])
        return n / np.linalg.norm(n, axis=1, keepdims=True)

    bounce = hemisphere_rays_from_hits(rays, want, normals, 8)
    hits, _, st = emul_cast(w, lv, t.verts, bounce, 0)
    rep = O.compare_closest(hits, O.cast_rays(t.nodes, t.verts, bounce, mode=O.MODE_GPU), bounce, t.slot_to_tri, t.verts)
    assert rep["ok"], {k_: v for k_, v in rep.items() if k_ != "rays"}
    shadow = bounce.copy()
    shadow["tMax"] = np.float32(0.2 * k)
    _, vis, _ = emul_cast(w, lv, t.verts, shadow, 1)
    assert np.array_equal(vis, O.any_rays(t.nodes, t.verts, shadow))


def test_wide8_emulated_traversal_on_small_scenes_against_brute_force():
    """Random rays (including rays starting inside boxes and axis-near directions) on small scenes:
    the emulated 8-wide traversal equals brute force over every triangle."""
    for args in [(8, 3, False, 5), (16, 12, True, 6), (24, 40, False, 7)]:
        s = P.generate_scene(*args)
        b = P.build_sbvh(s.tri_verts)
        w, lv = check_structure(b.nodes, len(b.verts))
        k = s.scale
        rays = random_rays(20_000, [-0.1 * k, -0.1 * k, -0.05 * k], [1.1 * k, 1.1 * k, 0.5 * k], args[3], tmin=1e-4)
        near_axis = rays[::7].copy()
        near_axis["dir"][:, 0] = np.float32(1e-7)
        d = near_axis["dir"]
        near_axis["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        rays = np.concatenate([rays, near_axis])
        hits, _, _ = emul_cast(w, lv, b.verts, rays, 0)
        bf = O.brute_closest(b.verts, rays, mode=O.MODE_GPU)
        rep = O.compare_closest(hits, bf, rays, b.slot_to_tri, b.verts)
        assert rep["ok"], (args, {k_: v for k_, v in rep.items() if k_ != "rays"})


def test_wide8_refuses_trees_whose_boxes_do_not_nest():
    s, b = built_scene("c1_64_100")
    nodes = b.nodes.copy()
    inner = np.nonzero((nodes["iData"][:, 2] == 0))[0]
    n = int(inner[1])
    child = int(nodes["iData"][n, 0])
    nodes["fData"][child, 0] -= np.float32(1.0)   # a grandchild box reaching outside its parent's box
    with pytest.raises(P.PheError) as e:
        P.wide8_build(nodes, len(b.verts))
    assert "inside its parent" in str(e.value)
