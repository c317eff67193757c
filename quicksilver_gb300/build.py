"""Build the native library in-tree (no CMake, no pip install).

``libqsg.so`` = host front end (C++, g++) + CUDA tracking kernels (nvcc,
``-gencode arch=compute_103a,code=sm_103a``).  Output goes to
``quicksilver_gb300/lib/``.  Translation units are compiled in parallel and
only rebuilt when a source or header is newer than the object.
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
OUT = PKG / "lib"
OBJ = OUT / "obj"
INCLUDE = ROOT / "include"
LIB = OUT / "libqsg.so"

HOST_SOURCES = ["host/status.cc", "host/deck.cc", "host/problem.cc", "host/batch.cc"]
CUDA_SOURCES = ["track.cu", "cycle.cu", "sens.cu"]

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no contraction into FMA, so every FP64 rounding matches the
# reference's CPU build (which is compiled without contraction).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-Wno-unused-parameter"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqsg.so")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _headers() -> list[Path]:
    return list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in _headers())


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip() and os.environ.get("QSG_BUILD_VERBOSE"):
        sys.stderr.write(res.stderr)


def build(verbose: bool = False, ptxas_verbose: bool = False, verify_screen: bool = False,
          nvtx: bool = False, portable_math: bool = False) -> Path:
    """Compile every translation unit and link ``libqsg.so``; returns its path.

    ``verify_screen`` builds ``libqsg_verify.so`` instead: the facet search also
    evaluates every facet the FP32 screen skipped and raises QSG_DEV_SCREEN_MISS
    if FP64 would have accepted one (a test build; slower).  ``nvtx`` builds
    ``libqsg_nvtx.so``: the same library with NVTX ranges around its phases
    (-DQSG_NVTX).  ``portable_math`` builds ``libqsg_pm.so``: the tracking
    path's log / sin / cos are the portable functions of
    csrc/portable_math.h (-DQSG_PORTABLE_MATH), the ones the oracle and the
    reference can be switched to, so that all three track bit-identical
    trajectories.  Each loads with QSG_LIB=verify / nvtx / pm.
    """
    if verify_screen + nvtx + portable_math > 1:
        raise ValueError("one variant at a time")
    variant = "verify" if verify_screen else "nvtx" if nvtx else "pm" if portable_math else ""
    obj_dir = OBJ / variant
    lib = OUT / (f"libqsg_{variant}.so" if variant else "libqsg.so")
    obj_dir.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for rel in HOST_SOURCES:
        src = CSRC / rel
        obj = obj_dir / (Path(rel).stem + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append(["g++", *CXX_FLAGS, f"-I{INCLUDE}", f"-I{CSRC / 'host'}", "-c", str(src), "-o", str(obj)])
    for rel in CUDA_SOURCES:
        src = CSRC / rel
        obj = obj_dir / (Path(rel).stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, src):
            flags = list(NVCC_FLAGS)
            if ptxas_verbose:
                flags += ["-Xptxas", "-v"]
            if verify_screen:
                flags += ["-DQSG_VERIFY_SCREEN"]
            if nvtx:
                flags += ["-DQSG_NVTX"]
            if portable_math:
                flags += ["-DQSG_PORTABLE_MATH"]
            jobs.append([nvcc, *NVCC_ARCH, *flags, f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CSRC / 'host'}",
                         "-c", str(src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for fut in [ex.submit(_run, j) for j in jobs]:
                fut.result()
    if jobs or not lib.exists():
        cuda_lib = _cuda_home() / "lib64"
        if not cuda_lib.exists():
            cuda_lib = _cuda_home() / "lib"
        link = ["g++", "-shared", "-o", str(lib), *map(str, objs), f"-L{cuda_lib}",
                f"-Wl,-rpath,{cuda_lib}", "-lcudart", "-lpthread"]
        _run(link)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv, verify_screen="--verify-screen" in sys.argv,
          nvtx="--nvtx" in sys.argv, portable_math="--portable-math" in sys.argv)
