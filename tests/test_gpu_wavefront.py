"""GPU parity of the wavefront frame (primary -> shade + shadow -> bounce -> shade + shadow ->
resolve) and of the TAA resolve against the oracle. Tolerance: 1e-4 absolute per channel in linear
FP32 (the shading and sampling arithmetic is written so both sides agree bit for bit; the tolerance
covers documented near-ties in hit selection)."""
import math

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300.renderer import (READ_COLOR, READ_HISTORY, READ_RAW, READ_ROUGHNESS, READ_VELOCITY,
                                                   CudaTracerRenderer, make_lights, taa_resolve)
from oracle import oracle as O
from tests.helpers import C1_CAM, built_scene, cam_struct, device_empty, from_device, to_device

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _setup(name, res, lights_xyz, graph=False):
    s, b = built_scene(name)
    datas = b.slot_datas(s.datas)
    scene = P.Scene(b.nodes, b.verts, datas, s.materials)
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
    lights = make_lights(np.asarray(lights_xyz, np.float32) * np.float32(k), range_=1000.0 * k)
    r = CudaTracerRenderer(use_graph=graph)
    r.setStaticScene(scene)
    r.setTargetResolution(res)
    return s, b, datas, scene, cam, cam_pos, lights, r


def _compare(gpu, ref, what):
    d = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    bad = (d > TOL).any(axis=-1) if d.ndim == 3 else d > TOL
    frac = bad.mean()
    assert frac <= 1e-5, f"{what}: {bad.sum()} pixels off by more than {TOL} (max {d.max()})"
    return d.max()


@pytest.mark.parametrize("graph,fused,refill,window", [(False, False, 20, 0), (True, False, 0, 1024), (True, False, 32, 256),
                                                      (False, True, 20, 0), (True, True, 20, 4096)])
def test_frame_matches_oracle_small(graph, fused, refill, window):
    res = (320, 184)
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0), (0.1, 0.9, 1.0)], graph)
    r.set_pipeline(fused=fused, refill=refill, sort_window=window)
    r.set_seed(1234, 0)
    r.resetTAA()
    jit = P.halton_jitter(3)
    r.set_camera_def(cam_struct(cam), cam_pos, jit)
    r.render(lights)
    raw = r.read(READ_RAW)
    rough = r.read(READ_ROUGHNESS)
    counts = r.ray_counts()
    ref, ref_rough, ref_counts = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, res, jit, cam_pos,
                                                1234, 0)
    _compare(raw, ref, "raw frame")
    assert np.array_equal(rough, ref_rough)
    assert np.array_equal(counts, ref_counts.astype(np.uint64))
    assert raw[..., :3].max() > 0.01 and (raw[..., :3] > 0).mean() > 0.2


@pytest.mark.parametrize("graph", [False, True])
def test_shadow_schedules_give_the_same_frame(graph):
    """Primary shadows in order, beside the bounce pass (second stream / parallel graph branch) or merged
    with the bounce shadows into one pass: the same bytes frame after frame (TAA history included), and
    per-kernel timing reports one kernel per launch of each schedule."""
    res = (256, 160)
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0), (0.9, 0.2, 1.5)], graph)
    out = {}
    for sched in (0, 1, 2):
        r.set_shadow_schedule(sched)
        r.set_seed(77, 0)
        r.resetTAA()
        for f in range(3):
            r.set_camera_def(cam_struct(cam), cam_pos, P.halton_jitter(f))
            r.render(lights)
        out[sched] = (r.read(READ_RAW), r.read(READ_HISTORY), r.ray_counts())
    for sched in (1, 2):
        for a, b_ in zip(out[0], out[sched]):
            assert np.array_equal(a, b_), sched
    r.set_graph(False)
    for sched, kernels in ((0, 5), (1, 5), (2, 4)):
        r.set_shadow_schedule(sched)
        r.set_kernel_timing(True)
        r.render(lights)
        r.render(lights)
        ms, frames = r.kernel_times()
        assert len(ms) == kernels and frames == 2 and np.all(ms > 0), (sched, ms, frames)
        r.set_kernel_timing(False)
    with pytest.raises(P.PheError):
        r.set_shadow_schedule(3)


@pytest.mark.parametrize("graph", [False, True])
def test_wide_layout_frame_gives_the_binary_frame(graph):
    """Switching the scene to 4-wide or 8-wide nodes between frames (graph re-captured) renders the same
    frame."""
    res = (256, 160)
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph)
    out = []
    for layout in (0, 1, 0, 2, 0):
        scene.set_layout(layout)
        r.set_seed(5, 0)
        r.resetTAA()
        for f in range(2):
            r.set_camera_def(cam_struct(cam), cam_pos, P.halton_jitter(f))
            r.render(lights)
        out.append((r.read(READ_RAW), r.ray_counts()))
    for raw, counts in out[1:]:
        _compare(raw, out[0][0], "wide vs binary frame")     # same hits up to documented near-ties
        assert np.abs(counts.astype(np.int64) - out[0][1].astype(np.int64)).max() <= 2


def test_async_read_back_matches_the_blocking_read():
    """read_async copies each frame's result while later frames render (colour and history from the
    side of the frame parity they were written to, roughness through a snapshot); after read_wait
    every host image equals the blocking read of the same frame."""
    import torch
    res = (320, 184)
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph=True)
    frames = 5
    want = []
    r.set_seed(3, 0)
    r.resetTAA()
    for f in range(frames):
        r.set_camera_def(cam_struct(cam), cam_pos, P.halton_jitter(f))
        r.render(lights)
        want.append((r.read(READ_COLOR), r.read(READ_ROUGHNESS), r.read(READ_HISTORY)))
    got = [torch.empty((res[1], res[0], 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(frames)]
    hist = [torch.empty((res[1], res[0], 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(frames)]
    rough = np.empty((res[1], res[0]), np.float32)        # pageable destination works too
    r.set_seed(3, 0)
    r.resetTAA()
    for f in range(frames):
        r.set_camera_def(cam_struct(cam), cam_pos, P.halton_jitter(f))
        r.render(lights)
        r.read_async(got[f])                              # colour and history: copied in place
        r.read_async(hist[f], READ_HISTORY)
        if f == frames - 1:
            r.read_async(rough, READ_ROUGHNESS)           # single-buffered: copied through a snapshot
    r.read_wait()
    for f in range(frames):
        assert np.array_equal(got[f], want[f][0]), f
        assert np.array_equal(hist[f], want[f][2]), f
    assert np.array_equal(rough, want[-1][1])
    with pytest.raises(ValueError):
        r.read_async(np.empty(10, np.float32))


@pytest.mark.parametrize("src,dst,viewport", [((320, 184), (1280, 720), None), ((1920, 1080), (1280, 720), None),
                                               ((333, 201), (333, 201), None), ((320, 184), (640, 400), (300, 150)),
                                               ((64, 40), (7, 3), None)])
def test_scaling_pass_matches_oracle(src, dst, viewport):
    import torch
    from phantasyenginetestbed_gb300.renderer import scale
    rng = np.random.default_rng(src[0] + dst[0])
    img = rng.uniform(0, 1.2, (src[1], src[0], 4)).astype(np.float32)
    d_src = to_device(img)
    d_dst = device_empty(dst[0] * dst[1], np.dtype((np.float32, 4)))
    d_rgba = device_empty(dst[0] * dst[1] * 4, np.uint8)
    scale(src, d_src, dst, d_dst, d_rgba, viewport=viewport)
    torch.cuda.synchronize()
    got = from_device(d_dst, np.float32).reshape(dst[1], dst[0], 4)
    ref = O.scale(img, dst, viewport)
    assert np.array_equal(got, ref)
    rgba = from_device(d_rgba, np.uint8).reshape(dst[1], dst[0], 4)
    assert np.array_equal(rgba[..., :3], np.rint(np.clip(ref[..., :3], 0, 1) * 255).astype(np.uint8))
    assert np.all(rgba[..., 3] == 255)


# The resolve kernel covers 256 pixels per block of 128 threads (two pixels a thread); the ragged sizes
# leave 64, 192, 128 and 64 pixels in the last block, so some threads have no second pixel or none.
@pytest.mark.parametrize("graph,res", [(False, (256, 160)), (True, (256, 160)), (False, (72, 40)), (True, (120, 40)),
                                       (False, (136, 48)), (True, (8, 8))])
def test_moving_camera_velocity_and_taa_match_oracle(graph, res):
    """Camera motion: still, moving, rotating, then still again (the previous velocity still weighs in)
    and still twice (the direct path). Per frame the velocity is bit-identical to the oracle's and the
    raw frame, TAA colour and history agree with the oracle's TAA chain."""
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph)
    k = s.scale
    d0 = np.array(C1_CAM["dir"], np.float64)
    d1 = d0 + np.array([0.03, 0.0, 0.01])
    p0 = np.array(cam_pos, np.float64)
    path = [(p0, d0), (p0, d0), (p0 + [0.004 * k, 0.001 * k, 0.0], d0), (p0 + [0.008 * k, 0.0, 0.002 * k], d1),
            (p0 + [0.008 * k, 0.0, 0.002 * k], d1), (p0 + [0.008 * k, 0.0, 0.002 * k], d1)]
    r.set_seed(5, 0)
    r.resetTAA()
    hist = np.zeros((res[1], res[0], 4), np.float32)
    prev_cam, prev_vel = None, np.zeros((res[1], res[0], 2), np.float32)
    for f, (pos, d) in enumerate(path):
        up = np.cross(np.cross(d, np.array(C1_CAM["up"])), d)   # orthogonal to d, as generateCameraDef needs
        up = -up if up[2] < 0 else up
        cam_f = O.camera_def(pos, d, up, math.radians(60), res)
        jit = P.halton_jitter(f)
        r.set_camera_def(cam_struct(cam_f), pos, jit)
        r.render(lights)
        vel = np.zeros((res[1], res[0], 2), np.float32)
        ref, rough, _ = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam_f, res, jit, pos, 5, f,
                                       prev_cam=cam_f if prev_cam is None else prev_cam, velocity_out=vel)
        _compare(r.read(READ_RAW), ref, f"raw frame {f}")
        got_vel = r.read(READ_VELOCITY)
        assert np.array_equal(got_vel, vel), f
        assert (np.abs(vel).max() > 0) == (f in (2, 3)), f
        out_c, hist = O.taa(ref, hist, rough, vel, prev_vel)
        _compare(r.read(READ_COLOR), out_c, f"TAA colour {f}")
        _compare(r.read(READ_HISTORY), hist, f"TAA history {f}")
        prev_cam, prev_vel = cam_f, vel


def test_frame_full_resolution_and_taa_sequence():
    """The wavefront-frame configuration: 1920x1080, point light at (0.5, 0.5, 2.0) * scale, 8 frames
    with Halton(2,3) jitter and the TAA resolve on an FP32 RGBA history."""
    res = (1920, 1080)
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph=True)
    r.set_seed(99, 0)
    r.resetTAA()
    hist = np.zeros((res[1], res[0], 4), np.float32)
    frames = (0, 7)
    for f in range(8):
        jit = P.halton_jitter(f)
        r.set_camera_def(cam_struct(cam), cam_pos, jit)
        r.render(lights)
        if f in frames or f == 7:
            raw = r.read(READ_RAW)
            ref, ref_rough, _ = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, res, jit, cam_pos, 99, f)
            _compare(raw, ref, f"frame {f}")
        # TAA on the GPU's own frames (frame parity is checked above): the blend must match the oracle
        raw_f = r.read(READ_RAW)
        rough = r.read(READ_ROUGHNESS)
        oc, hist = O.taa(raw_f, hist, rough)
        gc = r.read(READ_COLOR)
        gh = r.read(READ_HISTORY)
        assert np.array_equal(gc, oc) and np.array_equal(gh, hist)
    assert np.all(hist[..., 3][hist[..., 3] > 0] == 8.0)


def test_taa_resolve_with_velocity_matches_oracle():
    import torch
    rng = np.random.default_rng(4)
    W, H = 97, 61
    cur = rng.uniform(0, 2, (H, W, 4)).astype(np.float32)
    hist = rng.uniform(0, 2, (H, W, 4)).astype(np.float32)
    hist[..., 3] = rng.integers(0, 9, (H, W)).astype(np.float32)
    vel = (rng.normal(size=(H, W, 2)) * 0.02).astype(np.float32)
    vel[::3] = 0.0
    pvel = (rng.normal(size=(H, W, 2)) * 0.02).astype(np.float32)
    rough = rng.uniform(0, 1, (H, W)).astype(np.float32)
    d = [to_device(a) for a in (cur, hist, vel, pvel, rough)]
    oc = device_empty(W * H, np.dtype((np.float32, 4)))
    oh = device_empty(W * H, np.dtype((np.float32, 4)))
    taa_resolve((W, H), d[0], d[1], oc, oh, d[2], d[3], d[4])
    torch.cuda.synchronize()
    ref_c, ref_h = O.taa(cur, hist, rough, vel, pvel)
    got_c = from_device(oc, np.float32).reshape(H, W, 4)
    got_h = from_device(oh, np.float32).reshape(H, W, 4)
    assert np.array_equal(got_c, ref_c)
    assert np.array_equal(got_h, ref_h)
    moved = (vel != 0).any(-1)
    assert moved.any() and (~moved).any()


def test_renderer_rejects_bad_configuration():
    s, b = built_scene("c1_64_100")
    no_data_scene = P.Scene(b.nodes, b.verts)
    r = CudaTracerRenderer()
    with pytest.raises(P.PheError):
        r.setStaticScene(no_data_scene)
    with pytest.raises(P.PheError):
        r.setTargetResolution((100, 64))   # not a multiple of 8
    with pytest.raises(P.PheError):
        r.render(make_lights([(0, 0, 1)]))  # no scene, no resolution


def test_postprocess_matches_oracle_and_writes_an_image(tmp_path):
    import torch
    from phantasyenginetestbed_gb300.renderer import postprocess, write_ppm
    rng = np.random.default_rng(8)
    W, H = 64, 40
    lin = rng.uniform(0, 3, (H, W, 4)).astype(np.float32)
    lin[0, :5, :3] = [[0, 0, 0], [0.0015, 0.0015, 0.0015], [1e-3, 0, 2], [100, 50, 1e4], [0.5, 0.5, 0.5]]
    d_lin = to_device(lin)
    d_disp = device_empty(W * H, np.dtype((np.float32, 4)))
    d_rgba = device_empty(W * H * 4, np.uint8)
    postprocess((W, H), d_lin, d_disp, d_rgba)
    torch.cuda.synchronize()
    disp = from_device(d_disp, np.float32).reshape(H, W, 4)
    ref = O.postprocess(lin)
    assert np.abs(disp - ref).max() <= TOL          # powf on both sides: a few ulp apart at most
    rgba = from_device(d_rgba, np.uint8).reshape(H, W, 4)
    want = np.rint(np.clip(ref, 0, 1) * 255).astype(np.int32)
    assert np.abs(rgba.astype(np.int32) - want).max() <= 1
    write_ppm(tmp_path / "frame.ppm", rgba)
    assert (tmp_path / "frame.ppm").stat().st_size == len(b"P6\n64 40\n255\n") + W * H * 3


def test_renderer_lifecycle_lights_resolutions_and_resets():
    """8 lights (the maximum), a resolution that shrinks (buffers reused) and grows again, TAA resets in
    the middle, async read-backs across a resize: every frame equals the oracle's frame for its
    parameters."""
    import torch
    s, b = built_scene("c1_64_100")
    datas = b.slot_datas(s.datas)
    scene = P.Scene(b.nodes, b.verts, datas, s.materials)
    k = s.scale
    pts = np.array([(0.5, 0.5, 2.0), (0.1, 0.9, 1.0), (0.9, 0.1, 1.5), (0.3, 0.3, 0.8), (0.7, 0.7, 1.2),
                    (0.2, 0.6, 2.5), (0.8, 0.4, 0.9), (0.5, 0.1, 1.8)], np.float32) * np.float32(k)
    lights8 = make_lights(pts, range_=1000.0 * k)
    lights8["radius"][::2] = 0.02 * k          # area lights: random offsets on the light disc
    r = CudaTracerRenderer(use_graph=True)
    r.setStaticScene(scene)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    pinned = torch.empty((96, 128, 4), dtype=torch.float32, pin_memory=True).numpy()
    for f, (res, nl, reset) in enumerate([((128, 96), 8, True), ((64, 48), 3, False), ((64, 48), 1, True),
                                          ((128, 96), 8, False)]):
        r.setTargetResolution(res)
        cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
        if reset:
            r.resetTAA()
        r.set_seed(40 + f, f)
        jit = P.halton_jitter(f)
        r.set_camera_def(cam_struct(cam), cam_pos, jit)
        r.render(lights8[:nl])
        raw = r.read(READ_RAW)
        ref, rough, counts = O.render_frame(b.nodes, b.verts, datas, s.materials, lights8[:nl], cam, res, jit,
                                            cam_pos, 40 + f, f)
        _compare(raw, ref, f"frame {f}")
        assert np.array_equal(r.ray_counts(), counts.astype(np.uint64))
        out = pinned[: res[1], : res[0]].copy()
        r.read_async(out)
        r.read_wait()
        assert np.array_equal(out, r.read(READ_COLOR))


def test_async_read_back_across_a_reallocation():
    """An in-place read-back still in flight when a larger frame makes the renderer reallocate its
    buffers lands intact: the reallocation waits for it."""
    import torch
    s, b = built_scene("c1_64_100")
    scene = P.Scene(b.nodes, b.verts, b.slot_datas(s.datas), s.materials)
    k = s.scale
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    lights = make_lights(np.array([(0.5, 0.5, 2.0)] * 8, np.float32) * np.float32(k), range_=1000.0 * k)
    r = CudaTracerRenderer(use_graph=True)
    r.setStaticScene(scene)
    small, big = (64, 48), (512, 384)
    r.setTargetResolution(small)
    r.set_seed(5, 0)
    r.resetTAA()
    r.set_camera_def(cam_struct(O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), small)), cam_pos,
                     P.halton_jitter(0))
    r.render(lights[:1])
    want_color, want_hist = r.read(READ_COLOR), r.read(READ_HISTORY)
    out = torch.empty((small[1], small[0], 4), dtype=torch.float32, pin_memory=True).numpy()
    hist = torch.empty((small[1], small[0], 4), dtype=torch.float32, pin_memory=True).numpy()
    r.read_async(out)
    r.read_async(hist, READ_HISTORY)
    r.setTargetResolution(big)              # more pixels and lights: new frame buffers
    r.resetTAA()
    r.set_camera_def(cam_struct(O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), big)), cam_pos,
                     P.halton_jitter(1))
    r.render(lights)
    r.read_wait()
    assert np.array_equal(out, want_color)
    assert np.array_equal(hist, want_hist)
    assert r.read(READ_COLOR).shape[:2] == (big[1], big[0])


def test_async_read_back_of_velocity_and_colour_with_a_moving_camera():
    """With the camera moving, the per-pixel velocity is stored on the frame's parity side like the TAA
    colour; read_async of both every frame, without waiting in between, equals the blocking reads of
    the same frames (the frame after next waits for each in-place copy)."""
    import torch
    res = (256, 160)
    s, b, datas, scene, cam, cam_pos, lights, r = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph=True)
    k = s.scale
    d0 = np.array(C1_CAM["dir"], np.float64)
    p0 = np.array(cam_pos, np.float64)
    path = [p0 + np.array([0.002 * k * f, 0.0005 * k * f, 0.0]) for f in range(6)]

    def cam_at(f):
        up = np.cross(np.cross(d0, np.array(C1_CAM["up"])), d0)
        up = -up if up[2] < 0 else up
        return cam_struct(O.camera_def(path[f], d0, up, math.radians(60), res))

    want = []
    r.set_seed(8, 0)
    r.resetTAA()
    for f in range(len(path)):
        r.set_camera_def(cam_at(f), path[f], P.halton_jitter(f))
        r.render(lights)
        want.append((r.read(READ_COLOR), r.read(READ_VELOCITY)))
    assert all(np.abs(v).max() > 0 for _, v in want[1:])
    col = [torch.empty((res[1], res[0], 4), dtype=torch.float32, pin_memory=True).numpy() for _ in path]
    vel = [torch.empty((res[1], res[0], 2), dtype=torch.float32, pin_memory=True).numpy() for _ in path]
    r.set_seed(8, 0)
    r.resetTAA()
    for f in range(len(path)):
        r.set_camera_def(cam_at(f), path[f], P.halton_jitter(f))
        r.render(lights)
        r.read_async(col[f])
        r.read_async(vel[f], READ_VELOCITY)
    r.read_wait()
    for f in range(len(path)):
        assert np.array_equal(col[f], want[f][0]), f
        assert np.array_equal(vel[f], want[f][1]), f


def _flight_plan(s, cam_pos):
    """A frame sequence with camera motion, a TAA reset and a light-count change (2 lights, then 1)."""
    k = s.scale
    d0 = np.array(C1_CAM["dir"], np.float64)
    d1 = d0 + np.array([0.03, 0.0, 0.01])
    p0 = np.array(cam_pos, np.float64)
    one = make_lights(np.asarray([(0.5, 0.5, 2.0)], np.float32) * np.float32(k), range_=1000.0 * k)
    two = make_lights(np.asarray([(0.5, 0.5, 2.0), (0.1, 0.9, 1.0)], np.float32) * np.float32(k), range_=1000.0 * k)
    moved = p0 + [0.008 * k, 0.0, 0.002 * k]
    # (camera position, direction, lights, reset TAA before the frame)
    return [(p0, d0, one, False), (p0, d0, one, False), (p0 + [0.004 * k, 0.001 * k, 0.0], d0, one, False),
            (moved, d1, two, False), (moved, d1, two, False), (moved, d1, two, True), (moved, d1, one, False),
            (p0, d0, one, False), (p0, d0, one, False)]


def _flight_frame(r, f, step, res, stream):
    pos, d, lights, reset = step
    if reset:
        r.resetTAA(stream=stream)
    up = np.cross(np.cross(d, np.array(C1_CAM["up"])), d)
    up = -up if up[2] < 0 else up
    cam_f = O.camera_def(pos, d, up, math.radians(60), res)
    r.set_camera_def(cam_struct(cam_f), pos, P.halton_jitter(f))
    r.render(lights, stream=stream)


@pytest.mark.parametrize("res", [(256, 160), (120, 40)])
def test_frames_in_flight_give_the_sequential_frames(res):
    """Two frames in flight (consecutive frames overlapping on the renderer's own streams) give, frame
    after frame, the bytes of the same sequence rendered one frame at a time: TAA colour read back
    asynchronously in place while later frames render, and, with blocking reads after every frame, raw
    colour, history, roughness, velocity and ray counts. Latency recording returns one positive figure
    per frame."""
    import torch
    s, b, datas, scene, cam, cam_pos, lights, seq = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph=True)
    pip = CudaTracerRenderer()
    pip.setStaticScene(scene)
    pip.setTargetResolution(res)
    pip.set_frames_in_flight(2)
    plan = _flight_plan(s, cam_pos)
    stream = torch.cuda.Stream()
    host = lambda: torch.empty((res[1], res[0], 4), dtype=torch.float32, pin_memory=True).numpy()
    # pass 1: only asynchronous in-place colour reads while the frames run (overlapped on `pip`)
    colours = {}
    for name, r in (("seq", seq), ("pip", pip)):
        r.set_seed(21, 0)
        r.resetTAA(stream=stream)
        if r is pip:
            r.set_latency_recording(True)
        colours[name] = [host() for _ in plan]
        for f, step in enumerate(plan):
            _flight_frame(r, f, step, res, stream)
            r.read_async(colours[name][f], READ_COLOR, stream=stream)
        r.read_wait()
    for f in range(len(plan)):
        assert np.array_equal(colours["seq"][f], colours["pip"][f]), f
    lat = pip.frame_latencies()
    pip.set_latency_recording(False)
    assert len(lat) == len(plan) and np.all(lat > 0), lat
    # pass 2: blocking reads of every output after every frame
    for name, r in (("seq", seq), ("pip", pip)):
        r.set_seed(22, 0)
        r.resetTAA(stream=stream)
    for f, step in enumerate(plan):
        got = []
        for r in (seq, pip):
            _flight_frame(r, f, step, res, stream)
            got.append([r.read(w, stream=stream) for w in (READ_COLOR, READ_HISTORY, READ_RAW, READ_ROUGHNESS,
                                                             READ_VELOCITY)] + [r.ray_counts(stream=stream)])
        for a, c in zip(*got):
            assert np.array_equal(a, c), f
    pip.join(stream)
    stream.synchronize()
    pip.set_frames_in_flight(1)   # back to one frame: the same renderer keeps rendering the sequence
    _flight_frame(pip, len(plan), plan[0], res, stream)
    _flight_frame(seq, len(plan), plan[0], res, stream)
    assert np.array_equal(pip.read(READ_COLOR, stream=stream), seq.read(READ_COLOR, stream=stream))


@pytest.mark.parametrize("res,graph,parts", [((256, 160), True, 2), ((256, 160), False, 2), ((120, 40), True, 2),
                                             ((8, 8), False, 2), ((256, 160), True, 3), ((120, 40), False, 4),
                                             ((64, 24), True, 4)])
def test_split_frames_give_the_whole_frames(res, graph, parts):
    """A frame split into parts (tile rows dealt round-robin to parts on their own streams, own queues over
    shared per-pixel buffers) gives the bytes of the whole frame through camera motion, a TAA reset and a
    light-count change: TAA colour, history, raw colour, roughness, velocity and ray counts. 8x8 has one
    tile row, so it renders whole; 64x24 has three, so four parts run as three."""
    import torch
    s, b, datas, scene, cam, cam_pos, lights, whole = _setup("c2_256_2000", res, [(0.5, 0.5, 2.0)], graph=graph)
    split = CudaTracerRenderer(use_graph=graph)
    split.setStaticScene(scene)
    split.setTargetResolution(res)
    split.set_frame_parts(parts)
    plan = _flight_plan(s, cam_pos)
    stream = torch.cuda.Stream()
    for r in (whole, split):
        r.set_seed(31, 0)
        r.resetTAA(stream=stream)
    for f, step in enumerate(plan):
        got = []
        for r in (whole, split):
            _flight_frame(r, f, step, res, stream)
            got.append([r.read(w, stream=stream) for w in (READ_COLOR, READ_HISTORY, READ_RAW, READ_ROUGHNESS,
                                                             READ_VELOCITY)] + [r.ray_counts(stream=stream)])
        for a, c in zip(*got):
            assert np.array_equal(a, c), f
    with pytest.raises(P.PheError):
        split.set_frames_in_flight(2)
    split.set_frame_parts(1)
    _flight_frame(split, len(plan), plan[0], res, stream)
    _flight_frame(whole, len(plan), plan[0], res, stream)
    assert np.array_equal(split.read(READ_COLOR, stream=stream), whole.read(READ_COLOR, stream=stream))


@pytest.mark.parametrize("mode", ["parts", "flight"])
def test_split_and_flight_frames_across_resolution_changes(mode):
    """Split frames (2 parts) and two frames in flight across resolution changes (the second one grows
    the buffers, the third and fourth keep them) give the bytes of the same frames rendered whole, one
    at a time."""
    import torch
    s, b, datas, scene, cam, cam_pos, lights, ref = _setup("c2_256_2000", (64, 48), [(0.5, 0.5, 2.0)], graph=True)
    r = CudaTracerRenderer(use_graph=True)
    r.setStaticScene(scene)
    r.setTargetResolution((64, 48))
    if mode == "parts":
        r.set_frame_parts(2)
    else:
        r.set_frames_in_flight(2)
    stream = torch.cuda.Stream()
    plan = _flight_plan(s, cam_pos)
    for x in (ref, r):
        x.set_seed(41, 0)
    f = 0
    for res in [(64, 48), (128, 96), (64, 48), (128, 96)]:
        for x in (ref, r):
            x.setTargetResolution(res)
            x.resetTAA(stream=stream)
        colours = {}
        for x, name in ((ref, "ref"), (r, "test")):
            for k in range(3):
                _flight_frame(x, f + k, plan[k], res, stream)
            colours[name] = [x.read(w, stream=stream) for w in (READ_COLOR, READ_HISTORY, READ_RAW)] + \
                            [x.ray_counts(stream=stream)]
        for a, c in zip(colours["ref"], colours["test"]):
            assert np.array_equal(a, c), res
        f += 3
