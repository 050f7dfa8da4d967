"""ctypes view of the C ABI in ``include/mhd_gpu.h`` (``_lib/libmhdgpu.so``).

The library is the product path: there is no CPU fallback.  ``load()`` raises
if the shared object is missing or cannot be opened.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field, fields
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIBPATH = PKG / "_lib" / "libmhdgpu.so"

# enums mirrored from mhd_gpu.h
RECON_PDM, RECON_TVD, RECON_WENO5, RECON_MPWENO5, RECON_TVD_MC = 1, 2, 3, 4, 5
STEP_AB2, STEP_RK2, STEP_RK3 = 1, 2, 3
BC_PERIODIC, BC_EVEN, BC_REFLECT, BC_OUTFLOW = 0, 1, 2, 3
FP64, FP32 = 0, 1
DT_REFERENCE, DT_CFL = 0, 1
EMF_LFM, EMF_YEE = 0, 1
ST_NAN, ST_NEG_RHO, ST_NEG_P, ST_CFL, ST_TIMEOUT, ST_CUDA_ERROR = 1, 2, 4, 8, 16, 32
E_OK, E_ARG, E_CUDA, E_NOMEM, E_TIMEOUT, E_STATE = 0, -1, -2, -3, -4, -5

EXPORTS = (
    "mhd_init", "mhd_init_mapped", "mhd_step", "mhd_step_n", "mhd_fetch", "mhd_diagnostics", "mhd_step_graph",
    "mhd_set_tau", "mhd_set_profiling", "mhd_last_timings", "mhd_free", "mhd_last_error", "mhd_set_wait_bound",
    "mhd_device_info",
    "mhd_debug_fluxes", "mhd_debug_emf", "mhd_ensemble_step", "mhd_ensemble_time", "mhd_time_steps",
    "mhd_diagnostics_noalloc", "mhd_checkpoint_save", "mhd_checkpoint_load",
    "mhd_autotune", "mhd_ensemble_autotune", "mhd_set_tiles", "mhd_tc_gemm_test",
    "mhd_mlp_create", "mhd_mlp_params", "mhd_mlp_set_norm", "mhd_mlp_set_data", "mhd_mlp_grad", "mhd_mlp_train",
    "mhd_mlp_forward", "mhd_mlp_apply", "mhd_step_corrected", "mhd_mlp_free",
)


class CParams(C.Structure):
    _fields_ = [
        ("nx0", C.c_int32), ("ny0", C.c_int32), ("nz0", C.c_int32),
        ("nord", C.c_int32), ("reconop", C.c_int32), ("stepop", C.c_int32),
        ("bc", C.c_int32 * 3), ("precision", C.c_int32), ("dt_mode", C.c_int32),
        ("tvd_shift", C.c_int32),
        ("gam", C.c_double), ("cfl", C.c_double), ("pdmb", C.c_double), ("eps", C.c_double),
        ("alpha", C.c_double), ("beta", C.c_double), ("tau", C.c_double),
        ("emf", C.c_int32), ("reserved", C.c_int32 * 7),
    ]


@dataclass
class Params:
    """Deck scalars handed to ``mhd_init`` (namelists of mhd3d3.f90:152-156).

    Defaults are the reference's deck values (mhd3d3.in) with one rank per
    axis: PDM needs nord=8; gam = 5/3 (mhd3d3.f90:51).
    """
    nx0: int
    ny0: int
    nz0: int
    nord: int = 8
    reconop: int = RECON_PDM
    stepop: int = STEP_RK2
    bc: tuple = (BC_PERIODIC, BC_PERIODIC, BC_PERIODIC)
    precision: int = FP64
    dt_mode: int = DT_REFERENCE
    tvd_shift: int = 0
    gam: float = 5.0 / 3.0
    cfl: float = 0.3
    pdmb: float = 4.0
    eps: float = 1.0e-8
    alpha: float = 2.0
    beta: float = 4.0
    tau: float = 2.0e-4
    emf: int = EMF_LFM

    @property
    def ng(self) -> int:
        return self.nord // 2

    @property
    def shape(self) -> tuple:
        return (self.nx0 + self.nord, self.ny0 + self.nord, self.nz0 + self.nord)

    def to_c(self) -> CParams:
        p = CParams()
        for f in fields(self):
            v = getattr(self, f.name)
            if f.name == "bc":
                p.bc = (C.c_int32 * 3)(*[int(b) for b in v])
            else:
                setattr(p, f.name, v)
        return p


_LIB = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Open libmhdgpu.so (building it first if absent) and declare signatures.
    The environment variable MHD_LIB selects another build of the library."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    env = os.environ.get("MHD_LIB")
    p = Path(path) if path else (Path(env) if env else LIBPATH)
    if not p.exists():
        from . import build as _b
        _b.build()
    if not p.exists():
        raise RuntimeError(f"libmhdgpu.so not found at {p}; the CUDA library is required")
    lib = C.CDLL(str(p))
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    lib.mhd_init.argtypes = [C.POINTER(CParams)] + [dp] * 11 + [C.POINTER(vp)]
    lib.mhd_init_mapped.argtypes = [C.POINTER(CParams)] + [dp] * 11 + [C.POINTER(vp)]
    lib.mhd_step.argtypes = [vp, dp, C.POINTER(C.c_uint32)]
    lib.mhd_set_wait_bound.argtypes = [C.c_double]
    lib.mhd_step_n.argtypes = [vp, C.c_int32, dp, C.POINTER(C.c_uint32)]
    lib.mhd_step_graph.argtypes = [vp, C.c_int32, dp, C.POINTER(C.c_uint32)]
    lib.mhd_fetch.argtypes = [vp] + [dp] * 11
    lib.mhd_diagnostics.argtypes = [vp, dp]
    lib.mhd_set_tau.argtypes = [vp, C.c_double]
    lib.mhd_set_profiling.argtypes = [vp, C.c_int32]
    lib.mhd_last_timings.argtypes = [vp, C.POINTER(C.c_float)]
    lib.mhd_free.argtypes = [vp]
    lib.mhd_last_error.restype = C.c_char_p
    lib.mhd_device_info.argtypes = [C.POINTER(C.c_int32)]
    lib.mhd_debug_fluxes.argtypes = [vp, dp]
    lib.mhd_debug_emf.argtypes = [vp, dp, dp, dp]
    lib.mhd_time_steps.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_float)]
    lib.mhd_ensemble_step.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.POINTER(C.c_uint32)]
    lib.mhd_ensemble_time.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.POINTER(C.c_float)]
    lib.mhd_checkpoint_save.argtypes = [vp, C.c_char_p]
    lib.mhd_autotune.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
    lib.mhd_set_tiles.argtypes = [vp, C.c_int32, C.c_int32]
    lib.mhd_tc_gemm_test.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
    fp = C.POINTER(C.c_float)
    lib.mhd_mlp_create.argtypes = [C.c_void_p, C.POINTER(vp)]
    lib.mhd_mlp_params.argtypes = [vp, C.c_void_p, C.c_void_p]
    lib.mhd_mlp_set_norm.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.mhd_mlp_set_data.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_int64]
    lib.mhd_mlp_grad.argtypes = [vp, C.c_int64, C.c_int32, C.c_void_p, fp]
    lib.mhd_mlp_train.argtypes = [vp, C.c_int32, C.c_int32, C.c_float, C.c_uint64, fp]
    lib.mhd_mlp_forward.argtypes = [vp, C.c_void_p, C.c_int64, C.c_void_p]
    lib.mhd_mlp_apply.argtypes = [vp, vp]
    lib.mhd_step_corrected.argtypes = [vp, vp, C.c_int32, dp, C.POINTER(C.c_uint32)]
    lib.mhd_mlp_free.argtypes = [vp]
    lib.mhd_ensemble_autotune.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
    lib.mhd_checkpoint_load.argtypes = [C.c_char_p, C.POINTER(vp)]
    lib.mhd_diagnostics_noalloc.argtypes = [C.POINTER(CParams)] + [vp] * 12 + [vp]
    for name in EXPORTS:
        if name != "mhd_last_error":
            getattr(lib, name).restype = C.c_int
    if path is None:
        _LIB = lib
    return lib


class MHDError(RuntimeError):
    """A C-ABI call returned a negative MHD_E_* code (kept in ``code``)."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


def check(lib, rc: int, what: str) -> None:
    if rc != 0:
        msg = lib.mhd_last_error()
        raise MHDError(f"{what} failed ({rc}): {msg.decode() if msg else ''}", rc)
