"""Test infrastructure only: pulls named __device__ functions out of the reference's CUDA kernel
sources at build time, so that oracle/ref_shading.cpp can compile the reference's own shading and
sampling code as host code. The kernels in those files use launch syntax, surfaces and curand, which
a host compiler cannot take, while the helper functions themselves are plain C++ over sfz vectors.

The output goes to oracle/_ref/ (git-ignored) and starts each function with a #line directive that
points back into the reference file, so compiler messages and the code read as the reference's.

    python oracle/ref_extract.py <reference root> <output .inc>
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

# (file relative to the reference root, functions defined there that the shading harness calls)
FUNCTIONS = [
    ("source/cuda_ray_tracer/kernels/MaterialKernel.cu",
     ["setToDummyRay", "shadeHit", "hemisphereToWorld", "clampToHemisphere", "sampleGgx", "sampleLambertian"]),
    ("source/cuda_ray_tracer/kernels/InterpretRayHitKernel.cu", ["retrieveTriData"]),
]


def extract(text: str, name: str) -> tuple[int, str]:
    """(1-based first line, source) of the __device__ function `name` defined in `text`."""
    lines = text.splitlines(keepends=True)
    pat = re.compile(r"__device__.*\b" + re.escape(name) + r"\s*\(")
    for i, line in enumerate(lines):
        if not pat.search(line):
            continue
        # From this line, the definition runs to the brace that closes the first '{' (no ';' before it).
        rest = "".join(lines[i:])
        brace = rest.find("{")
        if brace < 0 or ";" in rest[:brace]:
            continue
        depth = 0
        for j in range(brace, len(rest)):
            if rest[j] == "{":
                depth += 1
            elif rest[j] == "}":
                depth -= 1
                if depth == 0:
                    return i + 1, rest[:j + 1]
    raise SystemExit(f"ref_extract: no definition of {name}")


def main() -> int:
    if len(sys.argv) != 3:
        print(__doc__, file=sys.stderr)
        return 2
    root, out = Path(sys.argv[1]), Path(sys.argv[2])
    parts = ["// Generated by oracle/ref_extract.py from the reference sources; not committed.\n"]
    for rel, names in FUNCTIONS:
        text = (root / rel).read_text(errors="replace")
        for name in names:
            first, src = extract(text, name)
            parts.append(f'#line {first} "{rel}"\n{src}\n')
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text("".join(parts))
    return 0


if __name__ == "__main__":
    sys.exit(main())
