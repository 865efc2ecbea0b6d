"""Compile the sm_103a CUDA library in-tree (no cmake, no torch extension).

``python -m sph_fem_2d_cutting_gpu_gb300.build`` (or ``build()``) compiles
every translation unit under ``csrc/`` with nvcc in parallel and links
``sph_fem_2d_cutting_gpu_gb300/lib/libsphfem.so``.  Object files go to
``_build/``.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG.parent / "_build" / "sphfem"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libsphfem.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "--expt-relaxed-constexpr",
                     "-Xptxas", "-warn-spills"]
SOURCES = ["cells.cu", "interactions.cu", "interactions_mlp.cu", "actions.cu", "fem.cu", "context.cu", "toolsetup.cpp",
           "noalloc.cu", "mlp.cu", "mlp_host.cu", "wear.cu", "vtk.cpp", "persistent.cu"]
HEADERS = ["common.cuh", "physics.cuh", "state.cuh", "launch.cuh", "toolsetup.h", "mlp_host.h", "rigid.cuh", "async.cuh",
           "p1elem.h", "interact32.cuh", "mlp_warp.cuh", "cells.cuh", "fem.cuh", "tail.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the sm_103a library cannot be built")


def _newest_header() -> float:
    hs = [CSRC / h for h in HEADERS] + [PKG.parent / "include" / "sphfem.h"]
    return max(h.stat().st_mtime for h in hs)


def _compile(src: Path, obj: Path, extra: list[str]) -> tuple[str, str]:
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}\n{r.stdout}")
    return src.name, r.stderr


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    extra = list(extra or [])
    BUILD.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    hdr_time = _newest_header()
    jobs = []
    objs = []
    for s in SOURCES:
        src = CSRC / s
        obj = BUILD / (s + ".o")
        objs.append(obj)
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_time) or extra:
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for name, log in ex.map(lambda a: _compile(a[0], a[1], extra), jobs):
            if verbose and log.strip():
                print(f"[{name}]\n{log}", file=sys.stderr)
    newest_obj = max(o.stat().st_mtime for o in objs)
    if jobs or not LIB.exists() or LIB.stat().st_mtime < newest_obj:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
