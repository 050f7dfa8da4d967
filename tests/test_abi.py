"""CPU tests of the C-ABI boundary: the library loads, exports every entry
point that include/mhd_gpu.h declares, the ctypes parameter block matches the
C struct layout, and argument validation answers without touching a GPU."""
import ctypes as C
import re
import shutil
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import abi
from mhd3d_mpi_fortran_gb300.abi import CParams, Params

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mhd_gpu.h"


def declared():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mhd_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    for n in ("mhd_init", "mhd_step", "mhd_fetch", "mhd_free"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    if shutil.which("nm"):
        out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIBPATH)], capture_output=True,
                             text=True).stdout
        exported = set(re.findall(r" T (mhd_\w+)", out))
        assert set(declared()) <= exported


def test_params_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "mhd_gpu.h"
int main(void){
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(mhd_params), offsetof(mhd_params,bc),
         offsetof(mhd_params,gam), offsetof(mhd_params,tau), offsetof(mhd_params,tvd_shift),
         offsetof(mhd_params,emf));
  return 0; }
'''
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "t.c"
        c.write_text(src)
        exe = Path(d) / "t"
        subprocess.run([cc, "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
        vals = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()))
    assert vals == [C.sizeof(CParams), CParams.bc.offset, CParams.gam.offset, CParams.tau.offset,
                    CParams.tvd_shift.offset, CParams.emf.offset]


@pytest.mark.parametrize("bad", [dict(nord=7), dict(reconop=9), dict(stepop=0), dict(nord=6, reconop=1),
                                 dict(nx0=0), dict(bc=(0, 0, 7)), dict(gam=1.0), dict(tau=0.0)])
def test_init_rejects_bad_decks(bad):
    """mhd_init validates the deck before any CUDA call (safe without a GPU)."""
    lib = abi.load()
    kw = dict(nx0=8, ny0=8, nz0=8)
    kw.update(bad)
    prm = Params(**kw).to_c()
    dummy = np.zeros(16)
    dp = dummy.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    rc = lib.mhd_init(C.byref(prm), *([dp] * 11), C.byref(h))
    assert rc == abi.E_ARG
    assert h.value is None
    assert lib.mhd_last_error()


def test_null_handle_is_an_argument_error():
    lib = abi.load()
    assert lib.mhd_step(None, None, None) == abi.E_ARG
    assert lib.mhd_free(None) == abi.E_OK
