"""phe_batch_cast_noalloc, the batched launch for callers that cannot let a library allocate device
memory: an engine's renderer or a plugin host that owns every byte of device memory through its own
allocator and budget, and must not have cudaMalloc called behind its back (it takes memory outside
their accounting and can wait for the whole device). Its scratch lives in a fixed array inside the
library instead.

Checked through the C ABI on two calls in a row against the allocating entry point (phe_batch_create +
phe_batch_launch) and against the oracle, with a 4-wide or 8-wide scene in the table, empty batches, exactly the
largest accepted item count, and the size refusals. The file name sorts last so that pytest collects it
after every other test: a run that stops at the first failure has run all the others before it."""
import ctypes as C

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300 import native as N
from phantasyenginetestbed_gb300.batch import ANY, CLOSEST, Batch
from oracle import oracle as O
from tests.helpers import device_empty, from_device, random_rays, to_device

pytestmark = pytest.mark.gpu

MAX_ITEMS = 256
MAX_SCENES = 32


def _scenes(wide_second=0):
    out = []
    for args in [(16, 10, False, 61), (48, 40, True, 62)]:
        s = P.generate_scene(*args)
        b = P.build_sbvh(s.tri_verts)
        out.append((s, b, P.Scene(b.nodes, b.verts)))
    if wide_second:
        out[1][2].set_layout(wide_second)
    return out


def _items(scenes, sizes, seed):
    rng = np.random.default_rng(seed)
    items, host = [], []
    for i, n in enumerate(sizes):
        si = int(rng.integers(len(scenes)))
        kind = CLOSEST if i % 3 else ANY
        s = scenes[si][0]
        rays = random_rays(max(n, 1), [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], seed * 1000 + i)[:n]
        if kind == ANY:
            rays["tMax"] = np.float32(0.5 * s.scale)
        d_rays = to_device(rays) if n else device_empty(32, P.RAY_IN_DTYPE)
        d_out = device_empty(max(n, 1), P.RAY_HIT_DTYPE if kind == CLOSEST else np.uint8)
        items.append((si, kind, n, d_rays, d_out))
        host.append(rays)
    return items, host


def _noalloc(scenes, items):
    arr = (C.c_void_p * len(scenes))(*[x[2].handle.value for x in scenes])
    table = (N.BatchItem * max(1, len(items)))()
    for i, (si, kind, n, d_rays, d_out) in enumerate(items):
        table[i] = N.BatchItem(si, kind, n, 0, d_rays.data_ptr(), d_out.data_ptr())
    N.check(N.lib().phe_batch_cast_noalloc(arr, len(scenes), table, len(items), None), "phe_batch_cast_noalloc")


def _check_against_oracle(scenes, items, host, got, call):
    for (si, kind, n, _, _), g, rays in zip(items, got, host):
        if n == 0:
            continue
        b = scenes[si][1]
        if kind == CLOSEST:
            want = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
            rep = O.compare_closest(g[:16 * n].view(P.RAY_HIT_DTYPE), want, rays, b.slot_to_tri, b.verts)
            assert rep["ok"], (call, rep)
        else:
            assert np.array_equal(g[:n], O.any_rays(b.nodes, b.verts, rays)), call


@pytest.mark.parametrize("wide", [0, N.LAYOUT_WIDE4, N.LAYOUT_WIDE8], ids=["binary", "wide4_scene", "wide8_scene"])
def test_noalloc_matches_allocating_launch_and_oracle_on_two_calls(wide):
    import torch
    scenes = _scenes(wide_second=wide)
    for call, (sizes, seed) in enumerate([([1000, 33, 5000, 1, 0, 640, 2048], 1), ([4096, 7, 100, 0, 12000, 64], 2)]):
        items, host = _items(scenes, sizes, seed)
        _noalloc(scenes, items)
        torch.cuda.synchronize()
        got = [from_device(it[4], np.uint8).copy() for it in items]
        _check_against_oracle(scenes, items, host, got, call)
        for it in items:
            it[4].fill_(0xCD)
        Batch([x[2] for x in scenes], items, use_graph=False).launch()
        torch.cuda.synchronize()
        for (si, kind, n, _, d_out), g in zip(items, got):
            want = from_device(d_out, np.uint8)
            assert np.array_equal(g[:(16 if kind == CLOSEST else 1) * n], want[:(16 if kind == CLOSEST else 1) * n]), call
    for x in scenes:
        assert x[2].status() == 0


def test_noalloc_accepts_exactly_its_largest_item_count():
    import torch
    scenes = _scenes()
    sizes = [int(x) for x in np.random.default_rng(9).integers(0, 70, MAX_ITEMS)]
    for call in range(2):
        items, host = _items(scenes, sizes, 20 + call)
        _noalloc(scenes, items)
        torch.cuda.synchronize()
        got = [from_device(it[4], np.uint8).copy() for it in items]
        _check_against_oracle(scenes, items, host, got, call)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    scenes = _scenes()
    d = device_empty(32, P.RAY_IN_DTYPE)
    o = device_empty(32, P.RAY_HIT_DTYPE)
    items = [(0, CLOSEST, 32, d, o)] * (MAX_ITEMS + 1)
    with pytest.raises(P.PheError) as e:
        _noalloc(scenes, items)
    assert e.value.status == N.PHE_ERR_TOO_LARGE
    assert f"at most {MAX_ITEMS}" in str(e.value)
    many = [scenes[i % 2] for i in range(MAX_SCENES + 1)]
    with pytest.raises(P.PheError) as e:
        _noalloc(many, [(0, CLOSEST, 32, d, o)])
    assert e.value.status == N.PHE_ERR_TOO_LARGE
    assert f"at most {MAX_SCENES}" in str(e.value)
