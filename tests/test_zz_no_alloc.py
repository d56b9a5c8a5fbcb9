"""phe_batch_cast_noalloc, the batched launch for callers that cannot let a library allocate device
memory (they own all of it through their own allocator and budget): its scratch lives in a fixed
array inside the library. Checked through the C ABI against the allocating entry point
(phe_batch_create + phe_batch_launch) on two calls in a row. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300 import native as N
from phantasyenginetestbed_gb300.batch import ANY, CLOSEST, Batch
from oracle import oracle as O
from tests.helpers import device_empty, from_device, random_rays, to_device

pytestmark = pytest.mark.gpu


def _scenes():
    out = []
    for args in [(16, 10, False, 61), (48, 40, True, 62)]:
        s = P.generate_scene(*args)
        b = P.build_sbvh(s.tri_verts)
        out.append((s, b, P.Scene(b.nodes, b.verts)))
    return out


def _items(scenes, sizes, seed):
    rng = np.random.default_rng(seed)
    items, host = [], []
    for i, n in enumerate(sizes):
        si = i % len(scenes)
        kind = CLOSEST if i % 3 else ANY
        s = scenes[si][0]
        rays = random_rays(n, [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], seed * 1000 + i)
        if kind == ANY:
            rays["tMax"] = np.float32(0.5 * s.scale)
        items.append((si, kind, n, to_device(rays), device_empty(n, P.RAY_HIT_DTYPE if kind == CLOSEST else np.uint8)))
        host.append(rays)
    return items, host


def _noalloc(scenes, items):
    arr = (C.c_void_p * len(scenes))(*[x[2].handle.value for x in scenes])
    table = (N.BatchItem * len(items))()
    for i, (si, kind, n, d_rays, d_out) in enumerate(items):
        table[i] = N.BatchItem(si, kind, n, 0, d_rays.data_ptr(), d_out.data_ptr())
    N.check(N.lib().phe_batch_cast_noalloc(arr, len(scenes), table, len(items), None), "phe_batch_cast_noalloc")


def test_noalloc_matches_allocating_launch_on_two_calls():
    import torch
    scenes = _scenes()
    for call, (sizes, seed) in enumerate([([1000, 33, 5000, 1, 640, 2048], 1), ([4096, 7, 100, 12000, 64], 2)]):
        items, host = _items(scenes, sizes, seed)
        _noalloc(scenes, items)
        torch.cuda.synchronize()
        got = [from_device(it[4], np.uint8).copy() for it in items]
        for it in items:
            it[4].fill_(0xCD)
        Batch([x[2] for x in scenes], items, use_graph=False).launch()
        torch.cuda.synchronize()
        for (si, kind, n, _, d_out), g, rays in zip(items, got, host):
            want = from_device(d_out, np.uint8)
            if kind == CLOSEST:
                b = scenes[si][1]
                rep = O.compare_closest(g.view(P.RAY_HIT_DTYPE), want.view(P.RAY_HIT_DTYPE), rays, b.slot_to_tri, b.verts)
                assert rep["ok"] and rep["near_ties"] == 0, (call, rep)
            else:
                assert np.array_equal(g, want), call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    scenes = _scenes()
    d = device_empty(32, P.RAY_IN_DTYPE)
    o = device_empty(32, P.RAY_HIT_DTYPE)
    items = [(0, CLOSEST, 32, d, o)] * 257
    with pytest.raises(P.PheError) as e:
        _noalloc(scenes, items)
    assert e.value.status == N.PHE_ERR_TOO_LARGE
    assert "at most 256" in str(e.value)
