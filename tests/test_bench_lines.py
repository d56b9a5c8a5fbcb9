"""The committed frame line (no GPU): its roofline figures recompute from the committed ncu summaries, its
secondary runs agree with their own fields, and a failed secondary run is reported in place."""
import json
import pathlib
import re

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_frame_line_roofline_recomputes_from_profiles():
    import bench
    line = json.loads((ROOT / "profiles" / "bench_frame_1080p.json").read_text())
    ncu = json.loads((ROOT / "profiles" / "ncu_kernels.json").read_text())
    roof = line["roofline"]
    sms = int(re.search(r"x (\d+) SMs", roof["how"]).group(1))
    mhz = line["clocks"]["sm_mhz"]
    # the dominant kernel: its ncu warp instructions per ray x the live rays / (live time x SMs x clock)
    k = ncu[f"{roof['kernel']}/{line['frame']['node_layout']}"]
    assert k["bvh_builder"] == line["config"]["bvh_builder"]
    pas = line["passes"][roof["pass"]]
    ipc = k["warp_inst_per_ray"] * pas["rays"] / (pas["ms"] * 1e-3 * sms * mhz * 1e6)
    assert abs(ipc - roof["achieved"]) < 2e-3 and abs(ipc / 4.0 - roof["frac"]) < 1e-3
    # the whole frame: the three traversal kernels' instructions / (frame time x SMs x clock)
    fi = bench.frame_issue(line["frame"]["rays_by_pass"], line["ms_per_step"], line["clocks"], sms,
                           line["config"]["bvh_builder"], line["frame"]["node_layout"])
    assert fi["frac"] == roof["frame_issue"]["frac"]
    assert 0.0 < roof["frac"] <= 1.2 and 0.0 < fi["frac"] <= 1.2


def test_secondary_runs_in_the_saved_line_are_consistent():
    line = json.loads((ROOT / "profiles" / "bench_frame_1080p.json").read_text())
    sec = line["secondary"]
    assert set(sec) == {"batch", "large", "serve"} and not any("error" in v for v in sec.values())
    b = sec["batch"]
    assert abs(b["plain_64_launches"]["ms"] / b["batched_graph"]["ms"] - b["speedup_vs_plain"]) < 5e-3
    assert abs(b["rays"] / b["batched_graph"]["ms"] / 1e3 - b["batched_graph"]["Mrays_s"]) < 0.5
    sv = sec["serve"]
    assert sv["continuous"]["errors"] == 0 and sv["serial"]["errors"] == 0
    assert sv["continuous"]["requests"] == sv["serial"]["requests"] and sv["continuous"]["rays"] == sv["serial"]["rays"]
    assert abs(sv["continuous"]["Mrays_s"] / sv["serial"]["Mrays_s"] - sv["speedup"]) < 5e-3
    lg = sec["large"]
    for pas in ("diffuse_closest", "shadow_any"):
        assert abs((16 << 20) / lg[pas]["ms"] / 1e3 - lg[pas]["Mrays_s"]) < 0.5 * 16
        assert 0.0 < lg["hbm_frac"][pas] < 1.2


def test_secondary_failures_are_reported_in_place(monkeypatch):
    import bench

    def boom(*args, **kwargs):
        raise RuntimeError("no device")

    for name in ("measure_batch", "measure_large", "measure_serve"):
        monkeypatch.setattr(bench, name, boom)
    out = bench.secondary_measures()
    assert out == {k: {"error": "RuntimeError: no device"} for k in ("batch", "large", "serve")}
