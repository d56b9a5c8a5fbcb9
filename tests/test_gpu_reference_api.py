"""The reference-signature C++ launch API (include/phe_reference_api.hpp) driven by a C++ program
that builds its inputs as the reference's renderer does (texture objects over linear memory);
results compared with the oracle and with the reference's own fixture."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import phantasyenginetestbed_gb300 as P
from phantasyenginetestbed_gb300 import build as B
from oracle import oracle as O
from tests.helpers import C1_CAM, golden_scene, load_golden

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def test_binary(tmp_path_factory):
    lib = B.build()
    out = tmp_path_factory.mktemp("refapi") / "reference_api_test"
    subprocess.run([B._nvcc(), *B.ARCH, "-std=c++17", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/reference_api_test.cu"),
                    "-o", str(out), f"-L{lib.parent}", "-lphe_gb300", f"-Xlinker=-rpath,{lib.parent}"], check=True)
    return out


def test_reference_launch_api_matches_oracle(test_binary, tmp_path):
    g = load_golden("ref_c1.npz")
    s, nodes, verts, s2t = golden_scene("ref_c1.npz")
    rays = O.gen_primary(g["cam"], C1_CAM["res"])[::4].copy()
    (tmp_path / "nodes.bin").write_bytes(nodes.tobytes())
    (tmp_path / "verts.bin").write_bytes(verts.tobytes())
    (tmp_path / "rays.bin").write_bytes(rays.tobytes())
    res = (64, 48)
    (tmp_path / "camera.bin").write_bytes(np.asarray(g["cam"], np.float32).tobytes() + np.array(res, np.int32).tobytes())
    r = subprocess.run([str(test_binary), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    orc = O.cast_rays(nodes, verts, rays, mode=O.MODE_GPU)
    for name in ("closest.bin", "plain.bin"):
        got = np.frombuffer((tmp_path / name).read_bytes(), P.RAY_HIT_DTYPE)
        rep = O.compare_closest(got, orc, rays, s2t, verts)
        assert rep["ok"] and rep["near_ties"] <= 2, rep
    lit = np.frombuffer((tmp_path / "shadow.bin").read_bytes(), np.uint8)
    assert np.array_equal(lit, O.any_rays(nodes, verts, rays))
    prim = np.frombuffer((tmp_path / "primary.bin").read_bytes(), P.RAY_IN_DTYPE)
    want = O.gen_primary(g["cam"], res, order=1)
    assert np.array_equal(prim.view(np.uint8), want.view(np.uint8))
