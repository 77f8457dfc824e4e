"""Build recipes for the native libraries of bevy_hair_gb300.

* ``_lib/libhairgb.so``   -- the sm_103a CUDA pipeline behind ``include/hairgb.h``.
  ``raster.cu`` and ``filter.cu`` are compiled with ``-fmad=false`` because
  their float results decide integer outputs (pixel coordinates, quantised
  depth, coverage) that must be reproducible bit for bit.
* ``_lib/libhairbake.so`` -- the host-side hair-mesh baker (``include/hairgb_bake.h``).

Objects compile in parallel; nothing here needs cmake.  The libraries are
built in-tree and are git-ignored.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_COMMON = [
    GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
    f"-I{ROOT / 'include'}",
]
EXACT_FLAGS = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
# Translation units whose float arithmetic feeds integer outputs.
EXACT_UNITS = {"raster.cu", "filter.cu"}
# Shading colour is compared within a tolerance; its exact outputs (view
# distance, reconstructed position, decoded tangent) use explicitly rounded
# intrinsics, which -use_fast_math does not change.
FAST_UNITS = {"shade.cu"}
CUDA_UNITS = ["api.cu", "raster.cu", "shade.cu", "filter.cu", "receiver.cu", "surrogate.cu", "batch.cu"]
# Host-only C++ linked into libhairgb.so.  -ffp-contract=off keeps f32 results
# the same on x86-64 and AArch64 (GCC would otherwise fuse into FMAs on Arm).
HOST_UNITS = ["host_params.cpp"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libhairgb.so")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_cuda(verbose_ptxas: bool = False, force: bool = False) -> Path:
    """Compile and link libhairgb.so for sm_103a."""
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "hairgb.h"]
    nv = nvcc()
    jobs = []
    objs = []
    for unit in CUDA_UNITS:
        src = CSRC / unit
        obj = BUILD_DIR / (unit + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src, *headers]):
            continue
        flags = list(NVCC_COMMON)
        if unit in EXACT_UNITS:
            flags += EXACT_FLAGS
        elif unit in FAST_UNITS:
            flags.append("-use_fast_math")
        else:
            flags += ["-prec-div=true", "-prec-sqrt=true"]
        if verbose_ptxas:
            flags.append("-Xptxas=-v")
        jobs.append([nv, *flags, "-c", str(src), "-o", str(obj)])
    cxx = os.environ.get("CXX", "g++")
    for unit in HOST_UNITS:
        src = CSRC / unit
        obj = BUILD_DIR / (unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, ROOT / "include" / "hairgb.h"]):
            jobs.append([cxx, *HOST_FLAGS, f"-I{ROOT / 'include'}", "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    lib = LIB_DIR / "libhairgb.so"
    if force or jobs or _stale(lib, objs):
        _run([nv, GENCODE, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    return lib


def build_probe(force: bool = False) -> Path:
    """The benchmark's measurement probes (L2 atomic throughput)."""
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    src = CSRC / "probe.cu"
    lib = LIB_DIR / "libhairprobe.so"
    if force or _stale(lib, [src]):
        _run([nvcc(), *NVCC_COMMON, "-shared", "-o", str(lib), str(src), "-lcudart"])
    return lib


def build_bake(force: bool = False) -> Path:
    """Compile the host baker."""
    LIB_DIR.mkdir(exist_ok=True)
    src = CSRC / "bake.cpp"
    lib = LIB_DIR / "libhairbake.so"
    deps = [src, ROOT / "include" / "hairgb_bake.h", ROOT / "include" / "hairgb.h"]
    if force or _stale(lib, deps):
        cxx = os.environ.get("CXX", "g++")
        # -ffp-contract=off: the same bake on x86-64 and AArch64
        _run([cxx, "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-shared", "-o", str(lib),
              str(src)])
    return lib


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_cuda, False, force), ex.submit(build_bake, force), ex.submit(build_probe, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    import sys

    build_all(force="--force" in sys.argv)
    print("built", LIB_DIR)
