"""In-tree build of the GB300 shared library ``_lib/libmhdgpu.so``.

The translation units are compiled in parallel with nvcc for sm_103a and
linked into one C-ABI library (declared in ``include/mhd_gpu.h``):

* ``csrc/mhd_fp64.cu`` -- FP64 kernels, ``-fmad=false`` (reference rounding),
* ``csrc/mhd_fp32.cu`` -- FP32 kernels (FMA contraction on),
* ``csrc/mhd_metric_fp64.cu`` / ``mhd_metric_fp32.cu`` -- the same kernels in
  curvilinear metric mode,
* ``csrc/mhd_geom.cu`` -- FP64 metric terms from node coordinates (``-fmad=false``),
* ``csrc/mhd_mlp.cu`` -- BF16 tcgen05 kernels of the learned coarse-grid correction,
* ``csrc/mhd_api.cu``  -- host sequencing and the ``extern "C"`` entry points,
* ``csrc/mhd_noalloc.cu`` -- the allocation-free diagnostics entry point.

Usage: ``python -m mhd3d_mpi_fortran_gb300.build`` (or ``build()``).
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
OUT = PKG / "_lib"
BUILD = PKG / "_build"
LIB = OUT / "libmhdgpu.so"
ROOT = PKG.parent

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]

UNITS = {
    "mhd_fp64": ["-fmad=false"],
    "mhd_fp32": ["-fmad=true"],
    "mhd_metric_fp64": ["-fmad=false"],
    "mhd_metric_fp32": ["-fmad=true"],
    "mhd_geom": ["-fmad=false"],
    "mhd_mlp": [],
    "mhd_api": ["-Xcompiler", "-fopenmp"],
    "mhd_noalloc": ["-fmad=false"],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmhdgpu.so")
    return cand


def _sources_newer(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
    deps.append(ROOT / "include" / "mhd_gpu.h")
    deps.append(Path(__file__))
    return any(p.stat().st_mtime > t for p in deps)


def _compile(unit: str, extra: list[str], verbose: bool) -> Path:
    obj = BUILD / f"{unit}.o"
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(CSRC / f"{unit}.cu"), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link ``libmhdgpu.so`` if any source is newer; returns its path."""
    if not force and not _sources_newer(LIB):
        return LIB
    BUILD.mkdir(exist_ok=True)
    OUT.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-Xcompiler", "-fopenmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
