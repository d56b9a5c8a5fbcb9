"""The checked build (libphe_gb300_checked.so: the same sources with PHE_DEVICE_CHECKS=1, every node and
slot index tested against its array before it is read, an error bit instead of an out-of-bounds read)
passes the ray-cast, frame, batch and no-alloc batch parity tests with no error bit raised. Runs them in a child process that
loads the checked library."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
pytestmark = pytest.mark.gpu

SUBSET = ["tests/test_gpu_raycast.py", "tests/test_gpu_wavefront.py::test_frame_matches_oracle_small",
          "tests/test_gpu_wavefront.py::test_split_frames_give_the_whole_frames",
          "tests/test_gpu_wavefront.py::test_frames_in_flight_give_the_sequential_frames",
          "tests/test_gpu_textures.py::test_textured_frame_matches_oracle", "tests/test_gpu_batch.py",
          "tests/test_zz_no_alloc.py"]


def test_checked_build_passes_the_parity_tests():
    if os.environ.get("PHE_GB300_CHECKED") == "1":
        pytest.skip("already running on the checked build")
    from phantasyenginetestbed_gb300 import build as B
    lib = B.build(checked=True)
    env = dict(os.environ, PHE_GB300_CHECKED="1")
    probe = subprocess.run([sys.executable, "-c", "from phantasyenginetestbed_gb300 import native; "
                            "native.lib(); print(native.LIB_PATH)"], env=env, cwd=ROOT, capture_output=True,
                           text=True, timeout=300)
    assert probe.returncode == 0 and probe.stdout.strip() == str(lib), probe.stdout + probe.stderr
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-m", "gpu", "-p", "no:cacheprovider", *SUBSET],
                       env=env, cwd=ROOT, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
