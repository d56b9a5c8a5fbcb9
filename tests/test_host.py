"""Host-side parts (no GPU): the C-ABI library loads and exports every declared symbol, the SBVH
builder emits a valid reference-layout tree of the reference builder's quality, scene validation,
the BVH cache file format."""
import re
from pathlib import Path

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300 import native
from oracle import oracle as O
from tests.helpers import random_rays, slot_verts

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(phe_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = native.lib()
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.phe_version() >= 100


def test_binding_table_covers_header():
    names = set(declared_functions())
    assert set(native.SIGNATURES) <= names
    unbound = names - set(native.SIGNATURES)
    assert not unbound, sorted(unbound)


def sah(nodes):
    f = nodes["fData"].astype(np.float64)
    i = nodes["iData"]

    def area(lo, hi):
        d = np.maximum(hi - lo, 0)
        return 2 * (d[:, 0] * d[:, 1] + d[:, 1] * d[:, 2] + d[:, 2] * d[:, 0])

    a0, a1 = area(f[:, 0:3], f[:, 3:6]), area(f[:, 6:9], f[:, 9:12])
    w0 = np.where(i[:, 2] > 0, i[:, 2], 1)
    w1 = np.where(i[:, 3] > 0, i[:, 3], 1)
    lo = np.minimum(f[0, 0:3], f[0, 6:9])
    hi = np.maximum(f[0, 3:6], f[0, 9:12])
    return float((a0 * w0 + a1 * w1).sum() / area(lo[None], hi[None])[0])


def check_layout(b, tri_verts):
    nodes, verts, s2t = b.nodes, b.verts, b.slot_to_tri
    assert P.validate_bvh(nodes, len(verts)) == b.max_depth <= 64
    # every slot belongs to exactly one leaf; end markers on the last slot of each leaf
    owner = np.zeros(len(verts), np.int32)
    for c in (0, 1):
        leaf = nodes["iData"][:, 2 + c] > 0
        assert np.all(nodes["iData"][leaf, c] < 0)          # leaf indices are negated
        first = ~nodes["iData"][leaf, c]
        cnt = nodes["iData"][leaf, 2 + c]
        for f, k in zip(first, cnt):
            owner[f:f + k] += 1
            assert np.all(verts["v0"][f:f + k - 1, 3] == 0) and verts["v0"][f + k - 1, 3] == -1
        inner = ~leaf
        assert np.all(nodes["iData"][inner, c] > 0)         # children come after their parent
    assert np.all(owner == 1)
    # every input triangle is referenced; slot vertices copy the input triangle
    assert np.array_equal(np.unique(s2t), np.arange(len(tri_verts)))
    tv = tri_verts[s2t]
    assert np.array_equal(verts["v0"][:, :3], tv[:, 0:3]) and np.array_equal(verts["v2"][:, :3], tv[:, 6:9])
    # child boxes contain the triangles' clipped parts: every leaf box overlaps its triangles' boxes
    return True


@pytest.mark.parametrize("args", [(8, 4, False, 1), (24, 30, True, 2), (64, 100, False, 1)])
def test_sbvh_layout_and_determinism(args):
    s = P.generate_scene(*args)
    b1 = P.build_sbvh(s.tri_verts, threads=1)
    b8 = P.build_sbvh(s.tri_verts, threads=8)
    check_layout(b1, s.tri_verts)
    assert np.array_equal(b1.nodes.view(np.uint8), b8.nodes.view(np.uint8))
    assert np.array_equal(b1.slot_to_tri, b8.slot_to_tri)


def test_sbvh_single_and_two_triangles():
    for T in (1, 2, 3):
        tv = np.random.default_rng(T).uniform(0, 1, (T, 9)).astype(np.float32)
        b = P.build_sbvh(tv)
        check_layout(b, tv)
        rays = random_rays(500, [-1, -1, -1], [2, 2, 2], T)
        tris = np.zeros(T, P.TRI_VERTS_DTYPE)
        tris["v0"][:, :3], tris["v1"][:, :3], tris["v2"][:, :3] = tv[:, 0:3], tv[:, 3:6], tv[:, 6:9]
        bf = O.brute_closest(tris, rays)
        got = O.cast_rays(b.nodes, b.verts, rays)
        hit = got["triangleIndex"] != 0xFFFFFFFF
        assert np.array_equal(hit, bf["triangleIndex"] != 0xFFFFFFFF)
        assert np.array_equal(b.slot_to_tri[got["triangleIndex"][hit]], bf["triangleIndex"][hit])


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("name", ["c1_64_100", "c3_155k"])
def test_sbvh_quality_matches_reference_builder(name):
    """Same SAH cost (within 2%) and slot count (within 5%) as the reference builder, and the same
    closest hits over both trees."""
    s = P.standard_scene(name)
    b = P.build_sbvh(s.tri_verts)
    rn, rv, rs = O.ref_build_sbvh(s.tri_verts)
    assert abs(sah(b.nodes) - sah(rn)) <= 0.02 * sah(rn)
    assert abs(len(b.verts) - len(rv)) <= 0.05 * len(rv)
    rays = random_rays(20000, [0, 0, 0.02], [s.scale, s.scale, 0.3 * s.scale], 8)
    mine = O.cast_rays(b.nodes, b.verts, rays)
    ref = O.cast_rays(rn, rv, rays)
    hm = mine["triangleIndex"] != 0xFFFFFFFF
    hr = ref["triangleIndex"] != 0xFFFFFFFF
    assert np.array_equal(hm, hr)
    same = b.slot_to_tri[mine["triangleIndex"][hm]] == rs[ref["triangleIndex"][hr]]
    assert same.mean() > 0.999
    assert np.allclose(mine["t"][hm][~same], ref["t"][hr][~same], rtol=1e-6)


def test_validation_rejects_malformed_trees():
    s = P.generate_scene(8, 2, False, 3)
    b = P.build_sbvh(s.tri_verts)
    ok = b.nodes.copy()
    assert P.validate_bvh(ok, len(b.verts)) >= 1
    cases = []
    x = ok.copy(); x["iData"][0, 2] = -3; cases.append(x)                      # negative count
    x = ok.copy(); x["iData"][0, 2] = 5; x["iData"][0, 0] = ~(len(b.verts) - 2); cases.append(x)  # leaf past end
    x = ok.copy(); x["fData"][0, 1] = np.nan; cases.append(x)                  # NaN bounds
    inner = np.nonzero(ok["iData"][:, 2] == 0)[0]
    x = ok.copy(); x["iData"][inner[-1], 0] = 0; cases.append(x)               # cycle to the root
    for c in cases:
        with pytest.raises(P.PheError) as e:
            P.validate_bvh(c, len(b.verts))
        assert e.value.status == native.PHE_ERR_INVALID_SCENE
    # a chain deeper than the traversal stack
    depth = 70
    chain = np.zeros(depth, P.NODE_DTYPE)
    for k in range(depth):
        chain["fData"][k] = [0, 0, 0, 1, 1, 1, 0, 0, 0, 1, 1, 1]
        chain["iData"][k] = [~0, k + 1, 1, 0] if k + 1 < depth else [~0, ~1, 1, 1]
    with pytest.raises(P.PheError):
        P.validate_bvh(chain, 2)


def test_bvh_cache_round_trip(tmp_path):
    import ctypes as C
    s = P.generate_scene(8, 3, True, 4)
    b = P.build_sbvh(s.tri_verts)
    datas = b.slot_datas(s.datas)
    base = str(tmp_path / "scene").encode()
    L = native.lib()
    native.check(L.phe_bvh_cache_write(base, native.ptr(b.nodes), len(b.nodes), native.ptr(b.verts),
                                       native.ptr(datas), len(b.verts)), "write")
    nn, ns = C.c_uint32(), C.c_uint32()
    native.check(L.phe_bvh_cache_sizes(base, C.byref(nn), C.byref(ns)), "sizes")
    assert (nn.value, ns.value) == (len(b.nodes), len(b.verts))
    n2 = np.empty(nn.value, P.NODE_DTYPE)
    v2 = np.empty(ns.value, P.TRI_VERTS_DTYPE)
    d2 = np.empty(ns.value, P.TRI_DATA_DTYPE)
    native.check(L.phe_bvh_cache_read(base, native.ptr(n2), nn.value, native.ptr(v2), native.ptr(d2), ns.value), "read")
    assert n2.tobytes() == b.nodes.tobytes() and v2.tobytes() == b.verts.tobytes() and d2.tobytes() == datas.tobytes()
    assert (tmp_path / "scene_header.bin").stat().st_size == 56

    def read():
        native.check(L.phe_bvh_cache_read(base, native.ptr(n2), nn.value, native.ptr(v2), native.ptr(d2), ns.value),
                     "read")

    # one flipped bit in an array is caught by the header's checksum ...
    raw = bytearray((tmp_path / "scene_verts.bin").read_bytes())
    raw[len(raw) // 2] ^= 0x10
    (tmp_path / "scene_verts.bin").write_bytes(bytes(raw))
    with pytest.raises(P.PheError) as e:
        read()
    assert e.value.status == 2 and "checksum" in str(e.value)
    # ... and a cache without the header (as the reference writes them) is read unchecked
    (tmp_path / "scene_header.bin").unlink()
    read()
    assert v2.tobytes() == bytes(raw)
    # a header of other counts is refused
    native.check(L.phe_bvh_cache_write(base, native.ptr(b.nodes), len(b.nodes), native.ptr(b.verts),
                                       native.ptr(datas), len(b.verts)), "write")
    hdr = bytearray((tmp_path / "scene_header.bin").read_bytes())
    hdr[24] ^= 1                      # numNodes
    (tmp_path / "scene_header.bin").write_bytes(bytes(hdr))
    with pytest.raises(P.PheError):
        read()
    # the reference's only check: vertex and data counts agree
    (tmp_path / "scene_datas.bin").write_bytes(d2[:-1].tobytes())
    with pytest.raises(P.PheError):
        native.check(L.phe_bvh_cache_sizes(base, C.byref(nn), C.byref(ns)), "sizes")


def test_scene_generator_shapes():
    s = P.standard_scene("c2_256_2000")
    assert s.tri_verts.shape == (155072, 9)
    assert np.all(np.isfinite(s.tri_verts))
    assert s.tri_verts[:131072, [0, 3, 6]].min() == 0.0 and s.tri_verts[:131072, [0, 3, 6]].max() == 4.0
    a = s.materials["albedo"][:, :3]
    assert a.min() >= 0.2 and a.max() <= 0.8
    n = s.datas["n0"]
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-6)


def test_persistent_launch_size_limit_is_checked_before_any_device_work():
    """n above PHE_MAX_PERSISTENT_RAYS is refused on the host, before the scene or the device is
    touched (the handles below are never dereferenced)."""
    import ctypes as C
    from phantasyenginetestbed_gb300 import native
    L = native.lib()
    fake = C.c_void_p(0x1000)
    assert L.phe_cast_closest(fake, fake, fake, 0xFC000001, None) == 8
    assert L.phe_cast_any(fake, fake, fake, 0xFFFFFFFF, None, None) == 8
    assert "rays per launch" in L.phe_last_error().decode()


def test_bvh_cache_python_wrappers(tmp_path):
    s = P.generate_scene(8, 3, True, 5)
    b = P.build_sbvh(s.tri_verts)
    datas = b.slot_datas(s.datas)
    P.write_bvh_cache(tmp_path / "c", b, datas)
    nodes, verts, d2 = P.read_bvh_cache(tmp_path / "c")
    assert nodes.tobytes() == b.nodes.tobytes() and verts.tobytes() == b.verts.tobytes()
    assert d2.tobytes() == datas.tobytes()
    assert P.validate_bvh(nodes, len(verts)) == b.max_depth


def _tree_is_valid(nodes, num_slots, max_depth=64):
    """The validation rules restated: from the root, every inner child index in range and reached once,
    inner nodes shallower than max_depth, leaf ranges inside the slot array, counts >= 0, no NaN bound."""
    n = len(nodes)
    if n == 0 or num_slots == 0:
        return False
    seen = np.zeros(n, bool)
    seen[0] = True
    stack = [(0, 0)]
    while stack:
        i, d = stack.pop()
        for c in range(2):
            raw, count = int(nodes["iData"][i, c]), int(nodes["iData"][i, 2 + c])
            if count < 0 or np.isnan(nodes["fData"][i, 6 * c: 6 * c + 6]).any():
                return False
            if count > 0:
                if (~raw if raw < 0 else raw) + count > num_slots:
                    return False
            elif raw < 0 or raw >= n or seen[raw] or d + 1 >= max_depth:
                return False
            else:
                seen[raw] = True
                stack.append((raw, d + 1))
    return True


def test_validation_agrees_with_the_rules_on_random_corruptions():
    """Hundreds of trees with random index, count and bound corruptions (small, negative, huge and
    boundary values): phe_bvh_validate accepts exactly those the rules restated in Python accept, and
    never crashes. Scene upload and every kernel rely on it to keep their indexing in bounds."""
    s = P.generate_scene(8, 3, True, 5)
    b = P.build_sbvh(s.tri_verts)
    T, N = len(b.verts), len(b.nodes)
    rng = np.random.default_rng(17)
    specials = np.array([0, 1, -1, -2, N - 1, N, N + 1, T - 1, T, ~0, ~(T - 1), ~T, 2**31 - 1, -2**31], np.int64)
    accepted = rejected = 0
    for trial in range(600):
        x = b.nodes.copy()
        for _ in range(int(rng.integers(1, 4))):
            i = int(rng.integers(0, N))
            if rng.random() < 0.1:
                x["fData"][i, int(rng.integers(0, 12))] = np.nan
                continue
            f = int(rng.integers(0, 4))
            v = int(rng.choice(specials)) if rng.random() < 0.5 else int(rng.integers(-3 * N, 3 * N))
            x["iData"][i, f] = np.int32(np.int64(v).astype(np.int32))
        want = _tree_is_valid(x, T)
        try:
            P.validate_bvh(x, T)
            got = True
        except P.PheError as e:
            assert e.status == native.PHE_ERR_INVALID_SCENE
            got = False
        assert got == want, trial
        accepted += got
        rejected += not got
    assert accepted > 20 and rejected > 200, (accepted, rejected)
