"""Builds the in-tree CUDA library grid2grid_gb300/_lib/libgrid2grid_gb300.so.

Plain nvcc, one -gencode for sm_103a, translation units compiled in
parallel, static CUDA runtime linked into the shared library. No cmake and no
torch extension machinery: the library exposes only the C ABI of
include/grid2grid_gb300.h.

    python -m grid2grid_gb300.build            # build if sources changed
    python -m grid2grid_gb300.build --force
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "libgrid2grid_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3",
          "-I", INCLUDE, "-I", CSRC]
CU_FLAGS = ARCH + COMMON + ["-Xptxas", "-O3"]

SOURCES = ["g2g_capi.cpp", "g2g_server.cpp", "g2g_scalapack.cpp", "g2g_reorder.cpp",
           "g2g_exchange.cpp",
           "g2g_planner.cu",
           "g2g_scatter.cu",
           "g2g_scatter_256.cu", "g2g_scatter_512.cu", "g2g_scatter_256e.cu",
           "g2g_scatter_512e.cu", "g2g_noalloc.cu", "g2g_volume.cu",
           "g2g_tma.cu"]
HEADERS = ["g2g_internal.hpp", "g2g_launch.hpp", "g2g_host.hpp", "g2g_scatter_impl.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc()] + CU_FLAGS
    if verbose_ptxas and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    cmd += ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compiles and links the library if any source is newer than it."""
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, "grid2grid_gb300.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= _newest(deps)):
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-Xcompiler", "-fPIC", "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
