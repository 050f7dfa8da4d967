"""Allocation-free diagnostics entry point, checked against mhd_diagnostics.

mhd_diagnostics_noalloc serves callers that cannot allocate device memory
when they need the diagnostics (a driver whose device memory all belongs to
its own pool, a latency-critical loop that must not take the implicit
synchronisation of cudaMalloc/cudaFree, a process at its MPS/MIG memory cap).
It reads arrays the caller already holds on the device and keeps its scratch
in a fixed file-scope device array.  This file is collected last on purpose;
it passes alone in a fresh process and after the rest of the suite.

The test itself allocates the device buffers it hands over (through the CUDA
runtime); only the entry point under test must not allocate.
"""
import ctypes as C

import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics, MHDSolver, abi
from mhd3d_mpi_fortran_gb300.abi import Params, FP64

pytestmark = pytest.mark.gpu

NAMES = ("mass", "energy", "divb_max", "rho_min", "dt_cfl")


class Runtime:
    """Minimal CUDA runtime access for the test's own device buffers."""

    def __init__(self):
        self.rt = C.CDLL("libcudart.so.13")
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.rt.cudaDeviceSynchronize.argtypes = []
        self.bufs = []

    def put(self, a: np.ndarray) -> C.c_void_p:
        a = np.asfortranarray(a, dtype=np.float64)
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), a.nbytes) == 0
        assert self.rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0  # host -> device
        self.bufs.append(p)
        return p

    def empty(self, n: int) -> C.c_void_p:
        return self.put(np.full(n, np.nan))

    def get(self, p: C.c_void_p, n: int) -> np.ndarray:
        out = np.zeros(n)
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0  # device -> host
        return out

    def free(self):
        for p in self.bufs:
            self.rt.cudaFree(p)
        self.bufs = []


def _device_inputs(rt, fields, grid):
    names = ("rho", "vx", "vy", "vz", "p", "bi", "bj", "bk")
    return [rt.put(fields[k]) for k in names] + [rt.put(grid.dx), rt.put(grid.dy), rt.put(grid.dz)]


def _check(got, ref):
    for i, k in enumerate(NAMES):
        # the same tolerance as the GPU parity tests' diagnostics check
        assert got[i] == pytest.approx(ref[k], rel=1e-13, abs=1e-15), k


def test_noalloc_matches_mhd_diagnostics_on_two_calls():
    lib = abi.load()
    s = ics.orszag_tang_3d(20, seed=5, ny0=18, nz0=16)
    g = s.grid
    prm = Params(20, 18, 16, precision=FP64, tau=0.5 * ics.cfl_dt(s))
    rt = Runtime()
    try:
        with MHDSolver(prm, s) as solver:
            out = rt.empty(5)
            cp = prm.to_c()
            for call in range(2):
                solver.step(2)
                ref = solver.diagnostics()
                args = _device_inputs(rt, solver.fetch(), g)
                rc = lib.mhd_diagnostics_noalloc(C.byref(cp), *args, out, None)
                assert rc == 0, lib.mhd_last_error()
                _check(rt.get(out, 5), ref)
    finally:
        rt.free()


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = abi.load()
    cp = Params(8, 8, 2041).to_c()  # 2049 z planes with nord = 8
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.mhd_diagnostics_noalloc(C.byref(cp), *([dummy] * 11), dummy, None)
    assert rc == abi.E_ARG
    assert b"2048" in lib.mhd_last_error()
