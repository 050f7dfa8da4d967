"""ORACLE -- test infrastructure only (tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may use it; the product path never does).

ctypes wrapper of ``oracle/_build/libmhdoracle.so``: the C++ FP64
restatement of the reference's step (mhd3d3.f90 step/get/reconstruct/fill
routines), with the same init/step/fetch interface as
``mhd3d_mpi_fortran_gb300.solver.MHDSolver``.  Parity unpinned against a
reference binary (none can be built here); see oracle/mhd_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmhdoracle.so"
_DP = C.POINTER(C.c_double)
_lib = None


def build() -> Path:
    src = HERE / "mhd_oracle.cpp"
    hdr = HERE.parent / "include" / "mhd_gpu.h"
    if not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        from mhd3d_mpi_fortran_gb300.abi import CParams
        lib.oracle_init.restype = C.c_void_p
        lib.oracle_init.argtypes = [C.POINTER(CParams)] + [_DP] * 11
        lib.oracle_init_mapped.restype = C.c_void_p
        lib.oracle_init_mapped.argtypes = [C.POINTER(CParams)] + [_DP] * 11
        lib.oracle_volumes.argtypes = [C.c_void_p, _DP]
        lib.oracle_step.argtypes = [C.c_void_p, C.c_int, _DP, C.POINTER(C.c_uint32)]
        lib.oracle_fetch.argtypes = [C.c_void_p] + [_DP] * 11
        lib.oracle_fluxes.argtypes = [C.c_void_p, _DP]
        lib.oracle_emf.argtypes = [C.c_void_p, _DP, _DP, _DP]
        lib.oracle_diagnostics.argtypes = [C.c_void_p, _DP]
        lib.oracle_recon_line.argtypes = [C.POINTER(CParams), C.c_int, _DP, _DP, _DP]
        lib.oracle_free.argtypes = [C.c_void_p]
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_set_fused.argtypes = [C.c_void_p, C.c_int]
        _lib = lib
    return _lib


def threads() -> int:
    return load().oracle_threads()


def set_threads(n: int) -> None:
    """OpenMP thread count of the following oracle calls."""
    load().oracle_set_threads(int(n))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_DP)


class OracleSolver:
    def __init__(self, params, state, dx=None, dy=None, dz=None):
        self.lib = load()
        self.params = params
        g = state.grid
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in state.arrays()]
        self._cp = params.to_c()
        self.metric = getattr(state, "nodes", None) is not None
        if self.metric:
            nodes = [np.asfortranarray(a, dtype=np.float64) for a in state.nodes]
            self.h = self.lib.oracle_init_mapped(C.byref(self._cp), *[_ptr(a) for a in arrs],
                                                 *[_ptr(a) for a in nodes])
            return
        geo = [np.ascontiguousarray(g.dx if dx is None else dx, dtype=np.float64),
               np.ascontiguousarray(g.dy if dy is None else dy, dtype=np.float64),
               np.ascontiguousarray(g.dz if dz is None else dz, dtype=np.float64)]
        self.h = self.lib.oracle_init(C.byref(self._cp), *[_ptr(a) for a in arrs], *[_ptr(a) for a in geo])

    def set_fused(self, on: bool = True) -> None:
        """Fused mode of the following steps: one pass per face / edge family,
        reconstructions evaluated at the point of use, no intermediate arrays;
        the same results as the array passes, bit for bit."""
        if self.lib.oracle_set_fused(self.h, 1 if on else 0) != 0:
            raise RuntimeError("oracle_set_fused failed")

    def step(self, n: int = 1):
        tau = C.c_double()
        st = C.c_uint32()
        self.lib.oracle_step(self.h, int(n), C.byref(tau), C.byref(st))
        return tau.value, st.value

    def fetch(self) -> dict:
        nx, ny, nz = self.params.shape
        cs = (nx, ny, nz)
        out = {k: np.zeros(cs, order="F") for k in ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz")}
        out["bi"] = np.zeros((nx + 1, ny, nz), order="F")
        out["bj"] = np.zeros((nx, ny + 1, nz), order="F")
        out["bk"] = np.zeros((nx, ny, nz + 1), order="F")
        names = ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "bi", "bj", "bk")
        self.lib.oracle_fetch(self.h, *[_ptr(out[k]) for k in names])
        return out

    def diagnostics(self) -> dict:
        out = np.zeros(5)
        self.lib.oracle_diagnostics(self.h, _ptr(out))
        return dict(zip(("mass", "energy", "divb_max", "rho_min", "dt_cfl"), out.tolist()))

    def volumes(self) -> np.ndarray:
        """Cell volumes of a metric-mode oracle (ghost-inclusive)."""
        nx, ny, nz = self.params.shape
        out = np.zeros((nx, ny, nz), order="F")
        assert self.lib.oracle_volumes(self.h, _ptr(out)) == 0
        return out

    def fluxes(self) -> list:
        p = self.params
        sizes = [(p.nx0 + (d == 0), p.ny0 + (d == 1), p.nz0 + (d == 2)) for d in range(3)]
        n = sum(8 * int(np.prod(s)) for s in sizes)
        buf = np.zeros(n)
        self.lib.oracle_fluxes(self.h, _ptr(buf))
        out, off = [], 0
        for s in sizes:
            m = int(np.prod(s))
            out.append([buf[off + q * m: off + (q + 1) * m].reshape(s, order="F") for q in range(8)])
            off += 8 * m
        return out

    def emf(self):
        p = self.params
        sh = [(p.nx0 + (e != 0), p.ny0 + (e != 1), p.nz0 + (e != 2)) for e in range(3)]
        es = [np.zeros(s, order="F") for s in sh]
        self.lib.oracle_emf(self.h, *[_ptr(a) for a in es])
        return es

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def recon_line(params, f: np.ndarray):
    """Face states of a 1-D line (oracle_recon_line): fl[c], fr[c] at the low
    face of cell c for c in [4, n-4)."""
    lib = load()
    f = np.ascontiguousarray(f, dtype=np.float64)
    fl = np.zeros_like(f)
    fr = np.zeros_like(f)
    cp = params.to_c()
    lib.oracle_recon_line(C.byref(cp), len(f), _ptr(f), _ptr(fl), _ptr(fr))
    return fl, fr


os.environ.setdefault("OMP_PROC_BIND", "false")
