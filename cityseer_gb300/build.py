"""Builds libcsgpu.so (sm_103a) in-tree with nvcc.

The library is the product's native boundary: CUDA kernels plus the C-ABI declared in
include/cityseer_gb300.h.  Sources are compiled in parallel, one -gencode, and linked with the
static CUDA runtime so the library loads on machines without a GPU driver (calls then fail with
CS_ERR_CUDA instead of the import failing).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = BUILD_DIR / "libcsgpu.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = ["cs_primal.cu", "cs_dual.cu", "cs_cta.cu"]
CXX_SOURCES = ["cs_host.cpp"]
HEADERS = ["cs_common.cuh", "cs_sort.cuh", "cs_seed.cuh", "cs_cta.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcsgpu.so")


def _needs_build() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = [CSRC / f for f in CUDA_SOURCES + CXX_SOURCES + HEADERS]
    deps.append(PKG_DIR.parent / "include" / "cityseer_gb300.h")
    deps.append(Path(__file__))
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the CUDA extension if any source is newer than the library; returns its path."""
    if not force and not _needs_build():
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    inc = f"-I{PKG_DIR.parent / 'include'}"
    common = [
        "-O3",
        "-std=c++17",
        "--extended-lambda",
        "-Xcompiler",
        "-fPIC,-ffp-contract=off",
        inc,
    ]
    jobs = []
    for src in CUDA_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        jobs.append(
            [nvcc, ARCH, "-lineinfo", "-fmad=false", "-Xptxas", "-v" if verbose else "-O3", "-c", str(CSRC / src),
             "-o", str(obj)] + common
        )
    for src in CXX_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        jobs.append([nvcc, "-c", str(CSRC / src), "-o", str(obj)] + common)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for lg in logs:
            print(lg)
    objs = [str(BUILD_DIR / (s + ".o")) for s in CUDA_SOURCES + CXX_SOURCES]
    tmp = BUILD_DIR / "libcsgpu.so.tmp"
    run([nvcc, ARCH, "-shared", "-o", str(tmp)] + objs + ["-Xcompiler", "-fPIC"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force=True, verbose="-v" in sys.argv))
