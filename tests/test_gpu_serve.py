"""Serving loop: continuous batching of ray-query and render requests. Each result is identical alone
and in the mix; ray queries match the oracle; renders match the renderer object; admission respects
the memory budget; the serial baseline gives the same results."""
import math

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300.renderer import READ_COLOR, CudaTracerRenderer, make_lights
from phantasyenginetestbed_gb300.serve import REQ_ANY, REQ_CLOSEST, REQ_RENDER, Server, pinned
from oracle import oracle as O
from tests.helpers import C1_CAM, cam_struct, random_rays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes():
    out = []
    for args in [(32, 20, True, 71), (64, 60, False, 72)]:
        s = P.generate_scene(*args)
        b = P.build_sbvh(s.tri_verts)
        out.append((s, b, P.Scene(b.nodes, b.verts, b.slot_datas(s.datas), s.materials)))
    return out


def _requests(scenes, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(14):
        si = i % 2
        s = scenes[si][0]
        if i % 3 == 2:
            res = (int(rng.choice([64, 96, 128])), int(rng.choice([48, 64, 96])))
            k = s.scale
            cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
            cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
            lights = make_lights(np.array([[0.5, 0.5, 2.0], [0.2, 0.8, 1.0]], np.float32)[: 1 + i % 2] * np.float32(k),
                                 range_=1000.0 * k)
            reqs.append(("render", si, dict(res=res, spp=1 + i % 3, cam=cam, cam_pos=cam_pos, lights=lights, seed=100 + i)))
        else:
            n = int(rng.integers(1, 20000))
            rays = random_rays(n, [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], seed * 100 + i)
            kind = REQ_ANY if i % 4 == 1 else REQ_CLOSEST
            if kind == REQ_ANY:
                rays["tMax"] = np.float32(0.4 * s.scale)
            reqs.append(("rays", si, dict(rays=rays, kind=kind)))
    return reqs


def _prepare(req):
    """Pinned host buffers of a request (allocated before submission so that submits are quick)."""
    kind, si, a = req
    if kind == "render":
        return None, pinned((a["res"][1], a["res"][0], 4), np.float32)
    rays = pinned(len(a["rays"]), P.RAY_IN_DTYPE)
    rays[:] = a["rays"]
    return rays, pinned(len(rays) * (1 if a["kind"] == REQ_ANY else 16), np.uint8)


def _submit(server, ids, req, bufs=None):
    kind, si, a = req
    rays, out = bufs if bufs is not None else _prepare(req)
    if kind == "render":
        rid = server.submit_render(ids[si], a["res"], a["spp"], cam_struct(a["cam"]), a["cam_pos"], a["lights"], a["seed"], out)
    else:
        rid = server.submit_rays(ids[si], rays, out, a["kind"])
    return rid, out


def test_each_result_is_the_same_alone_and_in_the_mix(scenes):
    # a 200 ms batching window: the queries submitted together below all join one wave
    server = Server(render_slots=3, batch_window_us=200000)
    ids = [server.add_scene(x[2]) for x in scenes]
    reqs = _requests(scenes, 1)
    alone = []
    for q in reqs:
        rid, out = _submit(server, ids, q)
        st = server.wait(rid)
        assert st.status == 0 and st.rays > 0
        alone.append(out.copy())
    waves_before = server.stats()["waves"]
    bufs = [_prepare(q) for q in reqs]
    mixed = [_submit(server, ids, q, bb) for q, bb in zip(reqs, bufs)]   # all in flight together
    server.drain()
    waves = server.stats()["waves"] - waves_before
    assert waves == 1   # every query of the mix went into one batched launch
    for (rid, out), a in zip(mixed, alone):
        st = server.poll(rid)
        assert st is not None and st.status == 0
        assert np.array_equal(out.view(np.uint8), a.view(np.uint8))
    # ray queries against the oracle, renders against the renderer object
    for (kind, si, a), res in zip(reqs, alone):
        s, b, sc = scenes[si]
        if kind == "rays":
            if a["kind"] == REQ_ANY:
                assert np.array_equal(res, O.any_rays(b.nodes, b.verts, a["rays"]))
            else:
                rep = O.compare_closest(res.view(P.RAY_HIT_DTYPE), O.cast_rays(b.nodes, b.verts, a["rays"]), a["rays"],
                                        b.slot_to_tri, b.verts)
                assert rep["ok"], rep
        else:
            r = CudaTracerRenderer()
            r.setStaticScene(sc)
            r.setTargetResolution(a["res"])
            r.set_seed(a["seed"], 0)
            r.resetTAA()
            for f in range(a["spp"]):
                r.set_camera_def(cam_struct(a["cam"]), a["cam_pos"], P.halton_jitter(f))
                r.render(a["lights"])
            assert np.array_equal(r.read(READ_COLOR), res)
    server.close()


def test_budget_admission_and_serial_baseline(scenes):
    sc_bytes = sum(x[2].device_bytes() for x in scenes)
    # room for the scenes plus about two 20K-ray queries at a time
    server = Server(memory_budget=sc_bytes + 2 * 20000 * 48 + 4096, render_slots=1)
    ids = [server.add_scene(x[2]) for x in scenes]
    s = scenes[0][0]
    big = pinned(200000, P.RAY_IN_DTYPE)
    big[:] = random_rays(200000, [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], 3)
    with pytest.raises(P.PheError) as e:
        server.submit_rays(ids[0], big, pinned(200000 * 16, np.uint8))
    assert e.value.status == 5   # PHE_ERR_BUDGET
    queries = []
    for i in range(8):
        rays = pinned(20000, P.RAY_IN_DTYPE)
        rays[:] = random_rays(20000, [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], 10 + i)
        out = pinned(20000 * 16, np.uint8)
        queries.append((server.submit_rays(ids[0], rays, out), rays, out))
    server.drain()
    b = scenes[0][1]
    for rid, rays, out in queries:
        assert server.poll(rid).status == 0
        rep = O.compare_closest(out.view(P.RAY_HIT_DTYPE), O.cast_rays(b.nodes, b.verts, rays), rays, b.slot_to_tri, b.verts)
        assert rep["ok"], rep
    server.close()
    # the serial baseline returns the same bytes
    serial = Server(serial=True, render_slots=1)
    ids = [serial.add_scene(x[2]) for x in scenes]
    for rid, rays, out in queries[:3]:
        out2 = pinned(len(rays) * 16, np.uint8)
        serial.wait(serial.submit_rays(ids[0], rays, out2))
        assert np.array_equal(out2, out)
    serial.close()


def test_cancel_and_malformed_requests(scenes):
    """Host-side fault injection: a queued request is cancelled (its output is never written), an
    admitted one is not; unknown scene ids and empty queries are refused at submit; rays with NaN
    components or tMin > tMax go through the server and give the results of a direct cast."""
    import torch
    s, b, scene = scenes[1]
    server = Server(serial=True, render_slots=1)
    sid = server.add_scene(scene)
    k = s.scale
    res = (1920, 1080)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
    lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
    big = pinned((res[1], res[0], 4), np.float32)
    first = server.submit_render(sid, res, 16, cam_struct(cam), cam_pos, lights, 1, big)   # keeps the server busy
    rays = random_rays(5000, [0, 0, 0.02], [k, k, 0.4 * k], 91)
    rays["dir"][::7, 1] = np.nan
    rays["origin"][3::11, 0] = np.nan
    rays["tMin"][5::13] = rays["tMax"][5::13] = 0.25 * k          # empty interval
    rays["tMin"][6::13] = np.float32(0.5 * k)
    rays["tMax"][6::13] = np.float32(0.1 * k)                      # tMin > tMax
    h_rays = pinned(len(rays), P.RAY_IN_DTYPE)
    h_rays[:] = rays
    outs = []
    ids = []
    for _ in range(3):
        out = pinned(len(rays) * 16, np.uint8)
        out[:] = 0xAB
        outs.append(out)
        ids.append(server.submit_rays(sid, h_rays, out, REQ_CLOSEST))
    assert server.cancel(ids[2]) is True                           # still queued behind the render
    assert server.cancel(ids[2]) is True                           # cancelling twice is harmless
    with pytest.raises(P.PheError) as e:
        server.wait(ids[2])
    assert e.value.status == 11
    server.wait(first)
    server.wait(ids[0])
    server.wait(ids[1])
    assert server.cancel(ids[0]) is False                          # completed: nothing to cancel
    assert np.all(outs[2] == 0xAB)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(len(rays) * 16, dtype=torch.uint8, device="cuda")
    P.cast_closest(scene, d_rays, d_hits, len(rays))
    torch.cuda.synchronize()
    want = d_hits.cpu().numpy()
    assert np.array_equal(outs[0], want) and np.array_equal(outs[1], want)
    hits = want.view(P.RAY_HIT_DTYPE)
    assert np.all(hits["triangleIndex"][5::13] == 0xFFFFFFFF) and np.all(hits["triangleIndex"][6::13] == 0xFFFFFFFF)
    with pytest.raises(P.PheError) as e:
        server.submit_rays(sid + 5, h_rays, outs[2], REQ_CLOSEST)
    assert e.value.status == 7
    with pytest.raises(P.PheError) as e:
        server.submit_rays(sid, h_rays[:0], outs[2], REQ_CLOSEST)
    assert e.value.status == 1
    server.close()


def test_concurrent_submitters_and_cancellers(scenes):
    """Four host threads submit queries at once while a fifth cancels some of them: every request ends
    exactly once, as done (bytes equal to a direct cast) or cancelled (output untouched)."""
    import threading
    import torch
    s, b, scene = scenes[0]
    server = Server(max_in_flight=4)
    sid = server.add_scene(scene)
    k = s.scale
    rays = random_rays(3000, [0, 0, 0.02], [k, k, 0.4 * k], 77)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(len(rays) * 16, dtype=torch.uint8, device="cuda")
    P.cast_closest(scene, d_rays, d_hits, len(rays))
    torch.cuda.synchronize()
    want = d_hits.cpu().numpy()
    h_rays = pinned(len(rays), P.RAY_IN_DTYPE)
    h_rays[:] = rays
    lock = threading.Lock()
    subs = []

    def submitter(t):
        for i in range(12):
            out = pinned(len(rays) * 16, np.uint8)
            out[:] = 0x5A
            rid = server.submit_rays(sid, h_rays, out, REQ_CLOSEST)
            with lock:
                subs.append((rid, out))

    def canceller():
        cancelled = 0
        for _ in range(200):
            with lock:
                cand = [rid for rid, _ in subs[-4:]]
            for rid in cand:
                cancelled += server.cancel(rid)
        return cancelled

    threads = [threading.Thread(target=submitter, args=(t,)) for t in range(4)] + [threading.Thread(target=canceller)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    server.drain()
    done = cancelled = 0
    for rid, out in subs:
        try:
            server.wait(rid)
            assert np.array_equal(out, want)
            done += 1
        except P.PheError as e:
            assert e.status == 11 and np.all(out == 0x5A)
            cancelled += 1
        server.release(rid)
    assert done + cancelled == 48 and done > 0
    st = server.stats()
    assert st["pending"] == 0 and st["in_flight"] == 0
    server.close()


@pytest.mark.parametrize("serial", [True, False])
def test_drain_returns_after_every_request(scenes, serial):
    """drain() returns only once every submitted request is done: none polls as not ready afterwards,
    including the last request of the serial baseline, which its worker serves with the lock released
    while it waits for the GPU."""
    server = Server(serial=serial, render_slots=1)
    ids = [server.add_scene(x[2]) for x in scenes]
    s = scenes[0][0]
    for rep in range(3):
        subs = []
        for i in range(6):
            n = 2000 + 3000 * i
            rays = pinned(n, P.RAY_IN_DTYPE)
            rays[:] = random_rays(n, [0, 0, 0.02], [s.scale, s.scale, 0.4 * s.scale], 40 + 10 * rep + i)
            out = pinned(n * 16, np.uint8)
            subs.append((server.submit_rays(ids[i % 2], rays, out, REQ_CLOSEST), rays, out))
        server.drain()
        for rid, rays, out in subs:
            st = server.poll(rid)
            assert st is not None and st.status == 0, (rep, rid)
            server.release(rid)
    server.close()


def test_queries_pass_a_render_that_waits_for_a_slot(scenes):
    """With one render slot busy, a second render waits for it; ray queries submitted behind that render
    are admitted past it instead of waiting too, and the second render is admitted only once the first
    one has completed. The queries' results equal the oracle."""
    server = Server(render_slots=1)
    ids = [server.add_scene(x[2]) for x in scenes]
    s, b, _ = scenes[0]
    k = s.scale
    res = (1024, 1024)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = cam_struct(O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res))
    lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
    frames = [pinned((res[1], res[0], 4), np.float32) for _ in range(2)]
    queries = []
    for i in range(4):
        rays = pinned(5000, P.RAY_IN_DTYPE)
        rays[:] = random_rays(5000, [0, 0, 0.02], [k, k, 0.4 * k], 900 + i)
        queries.append((rays, pinned(5000 * 16, np.uint8)))
    r1 = server.submit_render(ids[0], res, 8, cam, cam_pos, lights, 5, frames[0])
    r2 = server.submit_render(ids[0], res, 8, cam, cam_pos, lights, 6, frames[1])
    qids = [server.submit_rays(ids[0], rays, out, REQ_CLOSEST) for rays, out in queries]
    server.drain()
    first, second = server.poll(r1), server.poll(r2)
    assert first.status == 0 and second.status == 0
    assert second.admitMs >= first.doneMs - 1e-3   # the one slot was busy until the first render completed
    behind = 0
    for qid, (rays, out) in zip(qids, queries):
        st = server.poll(qid)
        assert st is not None and st.status == 0
        if st.submitMs < first.doneMs:
            behind += 1
            assert st.admitMs < second.admitMs, (st.submitMs, st.admitMs, first.doneMs, second.admitMs)
        rep = O.compare_closest(out.view(P.RAY_HIT_DTYPE), O.cast_rays(b.nodes, b.verts, rays), rays,
                                b.slot_to_tri, b.verts)
        assert rep["ok"], rep
        server.release(qid)
    assert behind > 0
    server.release(r1)
    server.release(r2)
    server.close()


def test_render_on_a_scene_in_use_goes_first(scenes):
    """Scene affinity: when a render slot frees and the next pending render's scene is not being
    rendered by any slot, a later pending render on a scene that a slot is rendering is admitted first.
    R1 (long) and R2 (shorter) render scene 0 in the two slots; R3 (scene 1) and R4 (scene 0) wait. When
    R2 completes, R1 still renders scene 0, so R4 goes before R3. Both frames equal the same renders
    made alone."""
    server = Server(render_slots=2)
    ids = [server.add_scene(x[2]) for x in scenes]

    def render_args(si, res):
        k = scenes[si][0].scale
        cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
        cam = cam_struct(O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res))
        lights = make_lights(np.array([[0.5, 0.5, 2.0]], np.float32) * np.float32(k), range_=1000.0 * k)
        return cam, cam_pos, lights

    plan = [(0, (1920, 1080), 8), (0, (512, 512), 4), (1, (256, 256), 1), (0, (256, 256), 1)]
    outs = [pinned((res[1], res[0], 4), np.float32) for _, res, _ in plan]
    args = [render_args(si, res) for si, res, _ in plan]
    rids = [server.submit_render(ids[si], res, spp, a[0], a[1], a[2], 30 + i, outs[i])
            for i, ((si, res, spp), a) in enumerate(zip(plan, args))]
    server.drain()
    st = [server.poll(r) for r in rids]
    assert all(x.status == 0 for x in st)
    assert st[2].submitMs < st[1].doneMs and st[3].submitMs < st[1].doneMs   # both waited for a slot
    assert st[0].doneMs > st[1].doneMs                                       # R1 still rendered scene 0
    assert st[3].admitMs < st[2].admitMs, [(x.submitMs, x.admitMs, x.doneMs) for x in st]
    for i in (2, 3):   # the reordered renders give the frames they give alone
        si, res, spp = plan[i]
        rid = server.submit_render(ids[si], res, spp, args[i][0], args[i][1], args[i][2], 30 + i,
                                   alone := pinned((res[1], res[0], 4), np.float32))
        assert server.wait(rid).status == 0
        assert np.array_equal(alone, outs[i])
        server.release(rid)
    for r in rids:
        server.release(r)
    server.close()
