"""Build the in-tree CUDA library ``diffmpm_gb300/libdiffmpm_gb300.so`` for sm_103a.

The library is compiled with nvcc directly (no CMake): each ``csrc/*.cu`` file
becomes an object in parallel, then they are linked into one shared library
with the CUDA runtime linked statically.  Floating-point contraction is off on
both sides (``-fmad=false`` for device code, ``-ffp-contract=off`` for host
code) so that every multiply and add rounds separately, as the reference's
arithmetic does.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
ROOT = PKG.parent
INCLUDE = ROOT / "include"
LIB = PKG / "libdiffmpm_gb300.so"
BUILD_DIR = ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--extended-lambda",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build diffmpm_gb300")
    return cand


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(outputs: Path, inputs) -> bool:
    if not outputs.exists():
        return True
    t = outputs.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def build(verbose: bool = False, force: bool = False, extra_flags=()) -> Path:
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
