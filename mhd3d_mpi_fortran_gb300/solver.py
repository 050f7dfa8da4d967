"""Host-side mirror of the reference's step interface over the C ABI.

``MHDSolver`` is what a Python driver (or a test) uses in place of the
reference's module state + ``call step``:

    s = MHDSolver(params, state)      # end of initialization (mhd3d3.f90:3327-3377)
    tau, status = s.step()            # call step (mhd3d3.f90:3286)
    fields = s.fetch()                # arrays read by outputxyz / diag_* (3091-3109, 3143-3160)
    s.close()                         # termination (3936-3943)

All arrays are FP64, Fortran order, ghost-inclusive, exactly the reference's
module arrays.  The work runs in ``libmhdgpu.so`` on the current CUDA device;
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import Params, check
from .ics import State

_DP = C.POINTER(C.c_double)


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["F_CONTIGUOUS"], "FP64 Fortran-order array required"
    return a.ctypes.data_as(_DP)


def _f64(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def output_arrays(params) -> dict:
    """Fortran-ordered FP64 arrays of the shapes mhd_fetch fills for params."""
    nx, ny, nz = params.shape
    cs = (nx, ny, nz)
    out = {k: np.zeros(cs, order="F") for k in ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz")}
    out["bi"] = np.zeros((nx + 1, ny, nz), order="F")
    out["bj"] = np.zeros((nx, ny + 1, nz), order="F")
    out["bk"] = np.zeros((nx, ny, nz + 1), order="F")
    return out


class MHDSolver:
    def __init__(self, params: Params, state: State | None, dx=None, dy=None, dz=None, lib=None,
                 _handle=None):
        self.lib = lib or abi.load()
        self.params = params
        if _handle is not None:  # from a checkpoint
            self.h = _handle
            return
        g = state.grid
        self._keep = [_f64(a) for a in state.arrays()]
        self._cp = params.to_c()
        h = C.c_void_p()
        if getattr(state, "nodes", None) is not None:
            # curvilinear metric mode: bi/bj/bk hold face fluxes Phi = B.A
            self._geo = [_f64(a) for a in state.nodes]
            rc = self.lib.mhd_init_mapped(C.byref(self._cp), *[_ptr(a) for a in self._keep],
                                          *[_ptr(a) for a in self._geo], C.byref(h))
            check(self.lib, rc, "mhd_init_mapped")
        else:
            self._geo = [_f64(g.dx if dx is None else dx), _f64(g.dy if dy is None else dy),
                         _f64(g.dz if dz is None else dz)]
            rc = self.lib.mhd_init(C.byref(self._cp), *[_ptr(a) for a in self._keep],
                                   *[_ptr(a) for a in self._geo], C.byref(h))
            check(self.lib, rc, "mhd_init")
        self.h = h
        self._keep = None

    # -- stepping -------------------------------------------------------
    def step(self, n: int = 1, graph: bool = False):
        tau = C.c_double()
        st = C.c_uint32()
        fn = self.lib.mhd_step_graph if graph else self.lib.mhd_step_n
        rc = fn(self.h, int(n), C.byref(tau), C.byref(st))
        check(self.lib, rc, "mhd_step")
        return tau.value, st.value

    def step_async(self, n: int = 1):
        """Enqueue n steps without waiting (no tau/status readback)."""
        rc = self.lib.mhd_step_n(self.h, int(n), None, None)
        check(self.lib, rc, "mhd_step_n")

    def time_steps(self, n: int, graph: bool = False) -> float:
        """Device time (ms) of n steps between CUDA events on the solver's stream."""
        ms = C.c_float()
        rc = self.lib.mhd_time_steps(self.h, int(n), 1 if graph else 0, C.byref(ms))
        check(self.lib, rc, "mhd_time_steps")
        return ms.value

    def autotune(self, reps: int = 5) -> tuple:
        """Pick the fastest compiled launch shapes for this grid (mhd_autotune);
        returns (face-tile length, EMF shape: 4 or 8 = ei tile, 1 = slice streams)."""
        out = (C.c_int32 * 2)()
        check(self.lib, self.lib.mhd_autotune(self.h, int(reps), out), "mhd_autotune")
        return out[0], out[1]

    def set_tiles(self, face_tile: int, ei_tile: int):
        """Set the launch shapes directly (mhd_set_tiles)."""
        check(self.lib, self.lib.mhd_set_tiles(self.h, int(face_tile), int(ei_tile)), "mhd_set_tiles")

    def save(self, path: str):
        """Checkpoint everything a step depends on (mhd_checkpoint_save)."""
        check(self.lib, self.lib.mhd_checkpoint_save(self.h, str(path).encode()), "mhd_checkpoint_save")

    @classmethod
    def load(cls, path: str, params: Params):
        """Resume from a checkpoint written by save(); params must describe the same run."""
        lib = abi.load()
        h = C.c_void_p()
        check(lib, lib.mhd_checkpoint_load(str(path).encode(), C.byref(h)), "mhd_checkpoint_load")
        return cls(params, None, lib=lib, _handle=h)

    def set_tau(self, tau: float):
        check(self.lib, self.lib.mhd_set_tau(self.h, float(tau)), "mhd_set_tau")

    def set_profiling(self, on: bool):
        check(self.lib, self.lib.mhd_set_profiling(self.h, 1 if on else 0), "mhd_set_profiling")

    def timings(self):
        out = (C.c_float * 8)()
        check(self.lib, self.lib.mhd_last_timings(self.h, out), "mhd_last_timings")
        return dict(zip(("flux_x", "flux_y", "flux_z_update", "emf", "ct", "fill", "dt"), list(out)))

    # -- readback -------------------------------------------------------
    def output_arrays(self) -> dict:
        """Fortran-ordered FP64 arrays of the shapes mhd_fetch fills."""
        return output_arrays(self.params)

    def fetch(self, out: dict | None = None) -> dict:
        """The state as FP64 Fortran arrays (mhd_fetch); `out` (from
        output_arrays, or arrays of the same shapes and layout) is filled in
        place, as the Fortran driver's own module arrays are."""
        if out is None:
            out = self.output_arrays()
        for k, a in out.items():
            if a.dtype != np.float64 or not a.flags.f_contiguous:
                raise ValueError(f"fetch: {k} must be a Fortran-ordered float64 array")
        names = ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "bi", "bj", "bk")
        rc = self.lib.mhd_fetch(self.h, *[_ptr(out[k]) for k in names])
        check(self.lib, rc, "mhd_fetch")
        return out

    def diagnostics(self) -> dict:
        out = (C.c_double * 5)()
        check(self.lib, self.lib.mhd_diagnostics(self.h, out), "mhd_diagnostics")
        return dict(zip(("mass", "energy", "divb_max", "rho_min", "dt_cfl"), list(out)))

    def debug_fluxes(self) -> list:
        p = self.params
        sizes = [(p.nx0 + (d == 0), p.ny0 + (d == 1), p.nz0 + (d == 2)) for d in range(3)]
        n = sum(8 * int(np.prod(s)) for s in sizes)
        buf = np.zeros(n)
        check(self.lib, self.lib.mhd_debug_fluxes(self.h, buf.ctypes.data_as(_DP)), "mhd_debug_fluxes")
        out, off = [], 0
        for s in sizes:
            m = int(np.prod(s))
            out.append([buf[off + q * m: off + (q + 1) * m].reshape(s, order="F") for q in range(8)])
            off += 8 * m
        return out

    def debug_emf(self):
        p = self.params
        sh = [(p.nx0 + (e != 0), p.ny0 + (e != 1), p.nz0 + (e != 2)) for e in range(3)]
        es = [np.zeros(s, order="F") for s in sh]
        check(self.lib, self.lib.mhd_debug_emf(self.h, *[_ptr(a) for a in es]), "mhd_debug_emf")
        return es

    def close(self):
        if getattr(self, "h", None):
            self.lib.mhd_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ensemble_step(solvers: list, nsteps: int) -> int:
    """Advance independent grids together in one CUDA graph (mhd_ensemble_step):
    Cartesian PDM grids with the same RK stepper share one launch per kernel
    family; other ensembles get one graph branch per grid."""
    lib = solvers[0].lib
    arr = (C.c_void_p * len(solvers))(*[s.h.value for s in solvers])
    st = C.c_uint32()
    check(lib, lib.mhd_ensemble_step(arr, len(solvers), int(nsteps), C.byref(st)), "mhd_ensemble_step")
    return st.value


def ensemble_time(solvers: list, nsteps: int) -> float:
    """Device time (ms) of nsteps ensemble steps (mhd_ensemble_time): CUDA
    events around the ensemble graph on the stream that carries it."""
    lib = solvers[0].lib
    arr = (C.c_void_p * len(solvers))(*[s.h.value for s in solvers])
    ms = C.c_float()
    check(lib, lib.mhd_ensemble_time(arr, len(solvers), int(nsteps), C.byref(ms)), "mhd_ensemble_time")
    return ms.value


def ensemble_autotune(solvers: list, reps: int = 5) -> tuple:
    """Pick the fastest launch shapes for a batched ensemble (mhd_ensemble_autotune)."""
    lib = solvers[0].lib
    arr = (C.c_void_p * len(solvers))(*[s.h.value for s in solvers])
    out = (C.c_int32 * 2)()
    check(lib, lib.mhd_ensemble_autotune(arr, len(solvers), int(reps), out), "mhd_ensemble_autotune")
    return out[0], out[1]
