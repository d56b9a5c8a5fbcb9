"""Maximum sizes, checked through size-independent properties.

* One persistent launch over 2^28 + 12,345 rays (8.6 GB of rays, 4.3 GB of hits: byte offsets far past
  2^32, ray indices near 2^28) made of copies of one 1M-ray period: every copy's results equal the first
  period's bit for bit, and the first period equals the oracle.
* The 8.6M-triangle scene (4.4M nodes, 13.3M slots: indices far past 2^22): a band of a 512x512 frame
  equals the oracle's band for the same rows, and 200K incoherent rays match the oracle.
"""
import math

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from oracle import oracle as O
from tests.helpers import C1_CAM, built_scene, cam_struct, random_rays

pytestmark = pytest.mark.gpu


def test_quarter_billion_ray_launch_is_periodic_and_matches_the_oracle():
    import torch
    s, b = built_scene("c1_64_100")
    scene = P.Scene(b.nodes, b.verts)
    period = 1 << 20
    rays = random_rays(period, [0, 0, 0.02], [1, 1, 0.3], 123)
    rays["tMax"][1::3] = np.float32(0.4)                    # some bounded rays for the any-hit pass
    copies = (1 << 8) + 1
    n = (1 << 28) + 12345
    d_period = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_rays = d_period.repeat(copies)[: n * 32]
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    P.cast_closest(scene, d_rays, d_hits, n)
    d_vis = torch.empty(n, dtype=torch.uint8, device="cuda")
    P.cast_any(scene, d_rays, d_vis, n)
    torch.cuda.synchronize()
    first = d_hits[: period * 16]
    full = (n // period) * period
    assert torch.equal(d_hits[: full * 16].view(-1, period * 16), first.expand(n // period, -1))
    assert torch.equal(d_hits[full * 16:], first[: (n - full) * 16])
    vfirst = d_vis[:period]
    assert torch.equal(d_vis[:full].view(-1, period), vfirst.expand(n // period, -1))
    assert torch.equal(d_vis[full:], vfirst[: n - full])
    got = first.cpu().numpy().view(P.RAY_HIT_DTYPE)
    orc = O.cast_rays(b.nodes, b.verts, rays, mode=O.MODE_GPU)
    rep = O.compare_closest(got, orc, rays, b.slot_to_tri, b.verts)
    assert rep["ok"] and rep["near_ties"] <= 2, rep
    assert np.array_equal(vfirst.cpu().numpy(), O.any_rays(b.nodes, b.verts, rays))
    assert scene.status() == 0
    del d_rays, d_hits, d_vis
    torch.cuda.empty_cache()


def test_large_scene_frame_band_and_incoherent_rays_match_the_oracle():
    from phantasyenginetestbed_gb300.renderer import READ_RAW, CudaTracerRenderer, make_lights
    import torch
    s, b = built_scene("c4_2048_20000")
    assert len(b.nodes) > (1 << 22) and len(b.verts) > (1 << 23)
    datas = b.slot_datas(s.datas)
    scene = P.Scene(b.nodes, b.verts, datas, s.materials)
    k = s.scale
    res = (512, 512)
    cam_pos = (0.5 * k, -0.3 * k, 0.6 * k)
    cam = O.camera_def(cam_pos, C1_CAM["dir"], C1_CAM["up"], math.radians(60), res)
    lights = make_lights(np.array([(0.5, 0.5, 2.0), (0.1, 0.1, 1.0)], np.float32) * np.float32(k), range_=1000.0 * k)
    r = CudaTracerRenderer(use_graph=True)
    r.setStaticScene(scene)
    r.setTargetResolution(res)
    r.set_seed(9, 0)
    r.resetTAA()
    jit = P.halton_jitter(2)
    r.set_camera_def(cam_struct(cam), cam_pos, jit)
    r.render(lights)
    raw = r.read(READ_RAW)
    band = (200, 264)
    ref, _, _ = O.render_frame(b.nodes, b.verts, datas, s.materials, lights, cam, res, jit, cam_pos, 9, 0, rows=band)
    d = np.abs(raw[band[0]:band[1]].astype(np.float64) - ref[band[0]:band[1]].astype(np.float64))
    assert (d > 1e-4).any(axis=-1).mean() <= 1e-4, d.max()
    assert raw[band[0]:band[1], :, :3].max() > 1e-3 and (raw[band[0]:band[1], :, :3] > 0).mean() > 0.2
    inc = random_rays(200_000, [0, 0, 0.02], [k, k, 0.3 * k], 321)
    d_rays = torch.from_numpy(inc.view(np.uint8)).cuda()
    d_hits = torch.empty(len(inc) * 16, dtype=torch.uint8, device="cuda")
    P.cast_closest(scene, d_rays, d_hits, len(inc))
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(P.RAY_HIT_DTYPE)
    orc = O.cast_rays(b.nodes, b.verts, inc, mode=O.MODE_GPU)
    rep = O.compare_closest(got, orc, inc, b.slot_to_tri, b.verts)
    assert rep["ok"] and rep["near_ties"] <= 20, rep
    assert scene.status() == 0
