"""Builds libgartus_gpu.so in-tree (gartus_gb300/_build/) for sm_103a.

Host code is compiled with -ffp-contract=off everywhere: GCC would otherwise fuse
multiply-adds on aarch64 and the f64 camera/BVH set-up would stop matching the
reference's unfused arithmetic.  The f64 device translation unit also disables fused
multiply-add (-fmad=false); the f32 one keeps it.
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
OUT = PKG / "_build"
LIB = OUT / "libgartus_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_COMMON = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math",
    "-I", str(PKG.parent / "include"),
]

UNITS = [
    ("api.cu", []),
    # The f32 throughput path: contracted multiply-adds and the hardware division and
    # square root (within 2 ulp; its parity is held to the f32 tolerances, not bit-exact).
    ("render_f32.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("render_f64.cu", ["-fmad=false"]),
    ("noalloc.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("denoise.cu", ["-fmad=true"]),
    ("lbvh.cu", ["-fmad=true"]),
]
CXX_UNITS = ["bvh_build.cpp", "scene_tables.cpp", "wide_bvh.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cuh", ".h", ".cpp")) + [
        PKG.parent / "include" / "gartus_gpu.h"
    ]


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _sources())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles every translation unit in parallel and links the shared library."""
    if not force and not _stale():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src, extra in UNITS:
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        jobs.append([nvcc, *ARCH, *NVCC_COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_UNITS:
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        jobs.append([os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off",
                     "-fno-fast-math", "-Wall", "-I", str(PKG.parent / "include"),
                     "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
