"""Test infrastructure only: stages the reference sources that the oracle harnesses compile into
baseline/_ref/ (git-ignored), so that the harnesses can be built wherever the repository goes,
including machines without the reference checkout.

Only the files the two harnesses need are copied, unchanged, with their paths relative to the
reference project root: the reference's CPU SBVH builder and castRay path (ray_tracer_common,
sbvh-stuff, the level/rendering headers they include, sfzCore headers and two of its sources) and
the headers / kernel sources whose shading functions oracle/ref_shading.cpp compiles as host code.
Nothing under baseline/_ref is committed or shipped; it is an install of the unmodified reference,
like the reference install that the benchmark's reference arm uses.

    python oracle/stage_reference.py [--from <reference root>]

The reference root defaults to $PHE_REFERENCE_ROOT, else /root/reference.
"""
from __future__ import annotations

import argparse
import os
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
DEST = ROOT / "baseline" / "_ref"
DEFAULT_SOURCE = "/root/reference"

# Directories copied whole (headers and sources of the CPU path) and single files.
TREES = [
    "externals/sfzCore/include",
    "source/phantasy_engine/ray_tracer_common",
    "source/phantasy_engine/sbvh-stuff",
    "source/phantasy_engine/level",
    "source/phantasy_engine/rendering",
]
FILES = [
    "LICENSE_PHANTASY_ENGINE",
    "LICENSE_SFZ_CORE",
    "externals/sfzCore/src/sfz/Assert.cpp",
    "externals/sfzCore/src/sfz/memory/Allocators.cpp",
    "source/cuda_ray_tracer/CudaPbr.cuh",
    "source/cuda_ray_tracer/CudaDeviceHelpers.cuh",
    "source/cuda_ray_tracer/CudaSfzVectorCompatibility.cuh",
    "source/cuda_ray_tracer/kernels/RayCastKernel.hpp",
    "source/cuda_ray_tracer/kernels/MaterialKernel.cu",
    "source/cuda_ray_tracer/kernels/InterpretRayHitKernel.cu",
    "source/phantasy_engine/screens/GameScreen.cpp",
]
# Extensions taken from the directories above (no binary assets).
EXTS = {".h", ".hpp", ".inl", ".cpp", ".cuh"}


def source_root(arg: str | None = None) -> Path | None:
    """The reference checkout to stage from, or None when none is present."""
    for cand in (arg, os.environ.get("PHE_REFERENCE_ROOT"), DEFAULT_SOURCE):
        if cand and (Path(cand) / "source" / "phantasy_engine").is_dir():
            return Path(cand)
    return None


def staged() -> bool:
    """True when baseline/_ref holds every file of the list."""
    return all((DEST / f).exists() for f in FILES) and all((DEST / t).is_dir() for t in TREES)


def stage(src: Path, dest: Path = DEST) -> int:
    n = 0
    for t in TREES:
        for p in sorted((src / t).rglob("*")):
            if p.is_file() and p.suffix in EXTS:
                q = dest / p.relative_to(src)
                q.parent.mkdir(parents=True, exist_ok=True)
                shutil.copy2(p, q)
                n += 1
    for f in FILES:
        q = dest / f
        q.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy2(src / f, q)
        n += 1
    (dest / "STAGED_FROM").write_text(f"unmodified reference files staged by oracle/stage_reference.py ({n} files)\n")
    return n


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--from", dest="src", default=None)
    a = ap.parse_args()
    src = source_root(a.src)
    if src is None:
        print("no reference checkout found (give --from or PHE_REFERENCE_ROOT)", file=sys.stderr)
        return 1
    print(f"staged {stage(src)} files from {src} into {DEST}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
