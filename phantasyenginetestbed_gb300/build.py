"""In-tree build of the native library libphe_gb300.so (CUDA kernels for sm_103a + C++ host code).

Every CUDA translation unit is compiled for sm_103a only, without fast-math and with FP contraction
off (-fmad=false): the kernels control rounding explicitly and must reproduce the host's IEEE results.
Host C++ is compiled with -ffp-contract=off for the same reason (gcc contracts by default on aarch64).
Translation units compile in parallel; the whole build takes well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libphe_gb300.so"
CHECKED_LIB = PKG / "libphe_gb300_checked.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-ftz=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-v", f"-I{ROOT / 'include'}",
]
CXX_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", f"-I{ROOT / 'include'}"]


def _cuda_include() -> str:
    """The toolkit's include directory (host files use its header-only NVTX)."""
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libphe_gb300.so")


def sources() -> tuple[list[Path], list[Path]]:
    cu = sorted((CSRC / "device").glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    return cu, cpp


def _compile(cmd: list[str], log: Path) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Builds libphe_gb300.so next to this file and returns its path. `checked` builds
    libphe_gb300_checked.so instead: the same sources with PHE_DEVICE_CHECKS=1 (device-side index
    checks in every traversal that set an error bit instead of reading out of bounds)."""
    nvcc = _nvcc()
    cu, cpp = sources()
    lib = CHECKED_LIB if checked else LIB
    build_dir = BUILD / "checked" if checked else BUILD
    defs = ["-DPHE_DEVICE_CHECKS=1"] if checked else []
    headers = list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.hpp")) + list((ROOT / "include").glob("*.h"))
    newest_dep = max(p.stat().st_mtime for p in cu + cpp + headers + [Path(__file__)])
    if lib.exists() and not force and lib.stat().st_mtime >= newest_dep:
        return lib
    build_dir.mkdir(parents=True, exist_ok=True)
    jobs = []
    objs = []
    for src in cu:
        obj = build_dir / (src.stem + ".cu.o")
        objs.append(obj)
        jobs.append(([nvcc, *NVCC_FLAGS, *defs, "-c", str(src), "-o", str(obj)], build_dir / (src.stem + ".cu.log")))
    cxx = os.environ.get("CXX", "g++")
    for src in cpp:
        obj = build_dir / (src.stem + ".cpp.o")
        objs.append(obj)
        jobs.append(([cxx, *CXX_FLAGS, *defs, f"-I{_cuda_include()}", "-c", str(src), "-o", str(obj)],
                     build_dir / (src.stem + ".cpp.log")))
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda j: _compile(*j), jobs))
    tmp = lib.with_suffix(".so.tmp")
    _compile([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"], build_dir / "link.log")
    os.replace(tmp, lib)
    if verbose:
        for log in sorted(build_dir.glob("*.cu.log")):
            sys.stdout.write(log.read_text())
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
