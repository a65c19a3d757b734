"""Build the sm_103a shared library ``libfddm_b200.so`` in-tree with nvcc.

The library is compiled from ``fastddm_gb300/csrc/*.cu`` for GB300 only
(``-gencode arch=compute_103a,code=sm_103a``); translation units compile in
parallel and are linked with a static CUDA runtime.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libfddm_b200.so"
LIB_PATH = PKG_DIR / LIB_NAME

# slowest translation units first, so the parallel build ends sooner
SOURCES = ["ddm_ff.cu", "ddm_f64.cu", "ddm_f32.cu", "fit_nv7.cu", "fit_nv6.cu", "fit_nv5.cu", "fit_nv4.cu", "fit_nv3.cu",
           "fit_nv2.cu", "fit_nv1.cu", "batch.cu", "capi.cu", "tables.cu", "tune.cu", "azavg.cu", "noalloc.cu", "sfio.cu",
           "tiffio.cpp", "postproc.cu", "dftstage.cu", "fit.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]
# per-file flags: the fits follow host arithmetic, which has no multiply-add contraction
FILE_FLAGS = {f"fit_nv{k}.cu": ["-fmad=false"] for k in range(1, 8)}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the GB300 kernels need the CUDA toolkit to build")
    return cand


def _inputs() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
                  + list(INCLUDE.glob("*.h")))


def is_stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _inputs())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile (if stale) and return the path of ``libfddm_b200.so``."""
    if not force and not is_stale():
        return LIB_PATH
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src: str) -> tuple[str, str]:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *FILE_FLAGS.get(src, []), *extra, "-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
        return str(obj), res.stderr

    workers = min(len(SOURCES), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_info:
        for _, log in results:
            if log:
                print(log)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *[o for o, _ in results]]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    p = build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(p)
