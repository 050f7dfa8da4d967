"""Allocation-free diagnostics entry point, checked against mhd_diagnostics.

mhd_diagnostics_noalloc serves callers that cannot allocate device memory
when they need the diagnostics (a driver whose device memory all belongs to
its own pool, a latency-critical loop that must not take the implicit
synchronisation of cudaMalloc/cudaFree, a process at its MPS/MIG memory cap).
It reads arrays the caller already holds on the device and keeps its scratch
in a fixed file-scope device array.

The file's name sorts it after every other test file, so pytest collects it
last: if it fails, a run that stops at the first failure (-x) has already run
the rest of the suite.  It depends on no state left by other tests and passes
alone in a fresh process as well as after them.

The test itself allocates the device buffers it hands over (through the CUDA
runtime); only the entry point under test must not allocate.
"""
import ctypes as C

import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics, MHDSolver, abi
from mhd3d_mpi_fortran_gb300.abi import Params, FP64, BC_OUTFLOW, BC_REFLECT

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
        self.rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        self.rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
        self.rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
        self.rt.cudaStreamDestroy.argtypes = [C.c_void_p]
        self.bufs = []

    def free_bytes(self) -> int:
        assert self.rt.cudaDeviceSynchronize() == 0
        f, t = C.c_size_t(), C.c_size_t()
        assert self.rt.cudaMemGetInfo(C.byref(f), C.byref(t)) == 0
        return f.value

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


def _deck(kind):
    """Periodic 3-D Orszag-Tang, or the magnetised blast between outflow or
    reflecting walls (whose ghost fills feed the min-rho and CFL reductions)."""
    if kind == "periodic":
        s = ics.orszag_tang_3d(20, seed=5, ny0=18, nz0=16)
        return s, Params(20, 18, 16, precision=FP64, tau=0.5 * ics.cfl_dt(s))
    s = ics.blast(16)
    bc = BC_OUTFLOW if kind == "outflow" else BC_REFLECT
    return s, Params(16, 16, 16, precision=FP64, bc=(bc,) * 3, tau=0.4 * ics.cfl_dt(s))


@pytest.mark.parametrize("kind", ["periodic", "outflow", "reflect"])
def test_noalloc_matches_mhd_diagnostics_on_two_calls(kind):
    """Two calls in a row, on the legacy default stream and then on a stream
    the caller created, each after two more steps: both match mhd_diagnostics
    of the same state."""
    lib = abi.load()
    s, prm = _deck(kind)
    rt = Runtime()
    stream = C.c_void_p()
    assert rt.rt.cudaStreamCreate(C.byref(stream)) == 0
    try:
        with MHDSolver(prm, s) as solver:
            out = rt.empty(5)
            cp = prm.to_c()
            for call, st in enumerate((None, stream)):
                solver.step(2)
                ref = solver.diagnostics()
                args = _device_inputs(rt, solver.fetch(), s.grid)
                rc = lib.mhd_diagnostics_noalloc(C.byref(cp), *args, out, st)
                assert rc == 0, lib.mhd_last_error()
                if st is not None:
                    assert rt.rt.cudaStreamSynchronize(st) == 0
                _check(rt.get(out, 5), ref)
    finally:
        rt.rt.cudaStreamDestroy(stream)
        rt.free()


def test_noalloc_warm_call_leaves_free_device_memory_unchanged():
    """After a first call (which may load the library's kernels), further calls
    change the device's free memory by nothing: the entry point allocates
    nothing, and its scratch is the static array."""
    lib = abi.load()
    s, prm = _deck("periodic")
    rt = Runtime()
    try:
        with MHDSolver(prm, s) as solver:
            args = _device_inputs(rt, solver.fetch(), s.grid)
            out = rt.empty(5)
            cp = prm.to_c()
            assert lib.mhd_diagnostics_noalloc(C.byref(cp), *args, out, None) == 0
            before = rt.free_bytes()
            for _ in range(3):
                assert lib.mhd_diagnostics_noalloc(C.byref(cp), *args, out, None) == 0, lib.mhd_last_error()
            after = rt.free_bytes()
            assert after == before, (before, after)
            _check(rt.get(out, 5), solver.diagnostics())
    finally:
        rt.free()


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = abi.load()
    cp = Params(8, 8, 2041).to_c()  # 2049 z planes with nord = 8
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.mhd_diagnostics_noalloc(C.byref(cp), *([dummy] * 11), dummy, None)
    assert rc == abi.E_ARG
    assert b"2048" in lib.mhd_last_error()
