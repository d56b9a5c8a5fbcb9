"""The committed frame line's roofline figures recompute from the committed ncu summaries (no GPU)."""
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
