"""Batched multi-scene persistent launch: every batch's result equals the oracle (closest-hit parity
rule / any-hit bit-exact) and equals the same batch cast alone with the plain per-batch launch, for
every autotuner candidate and with graph replay."""
import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300.batch import ANY, CLOSEST, ORDER_LARGEST_FIRST, Batch
from oracle import oracle as O
from tests.helpers import device_empty, from_device, random_rays, to_device

pytestmark = pytest.mark.gpu


def _scenes():
    out = []
    for args in [(16, 10, False, 51), (40, 30, True, 52), (64, 80, False, 53)]:
        s = P.generate_scene(*args)
        b = P.build_sbvh(s.tri_verts)
        out.append((s, b, P.Scene(b.nodes, b.verts)))
    return out


def _mix(scenes, sizes, seed):
    rng = np.random.default_rng(seed)
    items, host = [], []
    for i, n in enumerate(sizes):
        si = int(rng.integers(0, len(scenes)))
        kind = CLOSEST if rng.random() < 0.7 else ANY
        s = scenes[si][0]
        rays = random_rays(int(n), [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], seed * 100 + i)
        if kind == ANY:
            rays["tMax"] = np.float32(0.5 * s.scale)
        d_rays = to_device(rays)
        d_out = device_empty(int(n), P.RAY_HIT_DTYPE if kind == CLOSEST else np.uint8)
        items.append((si, kind, int(n), d_rays, d_out))
        host.append((si, kind, rays))
    return items, host


def _check(scenes, items, host):
    import torch
    torch.cuda.synchronize()
    for (si, kind, n, d_rays, d_out), (_, _, rays) in zip(items, host):
        s, b, _ = scenes[si]
        if kind == CLOSEST:
            got = from_device(d_out, P.RAY_HIT_DTYPE)
            rep = O.compare_closest(got, O.cast_rays(b.nodes, b.verts, rays), rays, b.slot_to_tri, b.verts)
            assert rep["ok"] and rep["near_ties"] <= 2, rep
        else:
            assert np.array_equal(from_device(d_out, np.uint8), O.any_rays(b.nodes, b.verts, rays))


def test_batched_launch_matches_oracle_and_plain():
    import torch
    scenes = _scenes()
    sizes = [1, 31, 32, 33, 1000, 5000, 17, 64, 20000, 3, 4096, 777]
    items, host = _mix(scenes, sizes, 3)
    batch = Batch([x[2] for x in scenes], items, use_graph=False)
    total, padded = batch.info()
    assert total == sum(sizes) and padded % 32 == 0 and padded >= total
    batch.launch()
    _check(scenes, items, host)
    # graph replay, other parameters
    for zero in items:
        zero[4].zero_()
    batch.set_params(block_size=256, order=ORDER_LARGEST_FIRST, use_graph=True)
    batch.launch()
    batch.launch()
    _check(scenes, items, host)
    # plain per-batch launches give the same bytes
    torch.cuda.synchronize()
    snapshot = [from_device(it[4], np.uint8).copy() for it in items]
    for (si, kind, n, d_rays, d_out) in items:
        if kind == CLOSEST:
            P.cast_closest(scenes[si][2], d_rays, d_out, n)
        else:
            P.cast_any(scenes[si][2], d_rays, d_out, n)
    torch.cuda.synchronize()
    for snap, it in zip(snapshot, items):
        assert np.array_equal(snap, from_device(it[4], np.uint8))


def test_autotuner_picks_a_valid_configuration():
    scenes = _scenes()
    items, host = _mix(scenes, [50000, 2000, 300, 10000, 64, 100000], 4)
    batch = Batch([x[2] for x in scenes], items)
    best, ms, table = batch.autotune(repeats=2)
    assert len(table) == 324 and ms > 0
    assert {r["layout"] for r in table} == {0, 1, 2}
    assert {r["stackShared"] for r in table} == {0, 16} and {r["sortWindow"] for r in table} == {0, 1024, 4096}
    assert best["blockSize"] in (64, 128, 256)
    assert ms == min(r["ms"] for r in table)
    for it in items:
        it[4].zero_()
    batch.launch()
    _check(scenes, items, host)


def test_sorted_and_shared_stack_launches_give_the_same_bytes():
    """Ray-sort granularity and the shared-memory stack depth change the order of work only: every
    window size (including windows larger than a batch and ragged last windows) and both stack depths
    write the same bytes as the plain launch, for closest and any hit."""
    import torch
    scenes = _scenes()
    sizes = [1, 31, 255, 256, 257, 1000, 4096, 5000, 20000, 0, 3, 777]
    items, host = _mix(scenes, sizes, 8)
    batch = Batch([x[2] for x in scenes], items, use_graph=False)
    batch.launch()
    torch.cuda.synchronize()
    want = [from_device(it[4], np.uint8).copy() for it in items]
    _check(scenes, items, host)
    for sw, sh, graph in ((256, 0, False), (1024, 16, False), (4096, 0, True), (0, 16, True), (2048, 16, True)):
        for it in items:
            it[4].fill_(0xCD)
        batch.set_params(block_size=64 if sh else 256, use_graph=graph, stack_shared=sh, sort_window=sw)
        batch.launch()
        batch.launch()
        torch.cuda.synchronize()
        for w, it in zip(want, items):
            assert np.array_equal(w, from_device(it[4], np.uint8)), (sw, sh)
    for s_ in scenes:
        assert s_[2].status() == 0
    with pytest.raises(P.PheError):
        batch.set_params(sort_window=100)
    with pytest.raises(P.PheError):
        batch.set_params(stack_shared=8)


def test_batch_rejects_bad_items():
    scenes = _scenes()
    d = device_empty(32, P.RAY_IN_DTYPE)
    o = device_empty(32, P.RAY_HIT_DTYPE)
    with pytest.raises(P.PheError):
        Batch([scenes[0][2]], [(1, CLOSEST, 32, d, o)])      # scene index out of range
    with pytest.raises(P.PheError):
        Batch([scenes[0][2]], [(0, 7, 32, d, o)])            # unknown kind


@pytest.mark.parametrize("graph", [False, True], ids=["direct", "graph"])
def test_update_right_after_a_launch_on_a_non_blocking_stream(graph):
    """phe_batch_update rewrites the item table in place while the launch before it may still read it, on
    a stream that is not ordered after the legacy default stream (torch's side streams are created
    non-blocking): the update waits for that launch and its upload is complete when it returns, so both
    launches give the oracle's results."""
    import torch
    scenes = _scenes()
    sizes = [20000, 5000, 777, 4096, 31]
    items_a, host_a = _mix(scenes, sizes, 11)
    items_b, host_b = _mix(scenes, sizes, 12)
    torch.cuda.synchronize()   # the rays' uploads ran on the default stream
    side = torch.cuda.Stream()
    batch = Batch([x[2] for x in scenes], items_a, use_graph=graph)
    for _ in range(2):
        for it in items_a + items_b:
            it[4].fill_(0xCD)
        torch.cuda.synchronize()
        batch.update(items_a)
        batch.launch(stream=side)
        batch.update(items_b)
        batch.launch(stream=side)
        side.synchronize()
        _check(scenes, items_a, host_a)
        _check(scenes, items_b, host_b)
    for s_ in scenes:
        assert s_[2].status() == 0
