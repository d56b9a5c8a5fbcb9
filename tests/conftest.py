import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native library and the oracle once per session (quick when up to date)."""
    from phantasyenginetestbed_gb300 import build as B
    from oracle import oracle as O
    B.build()
    O.build()
    yield
