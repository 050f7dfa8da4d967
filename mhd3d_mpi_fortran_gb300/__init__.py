"""GB300 (sm_103a) per-timestep ideal-MHD update of tiegcm/mhd3d_mpi_fortran.

The product is the C-ABI library ``_lib/libmhdgpu.so`` (``include/mhd_gpu.h``);
this package builds it in-tree and mirrors the reference's step interface in
Python (``MHDSolver``).  ``ics`` holds the initial-condition generators and
``deck`` the namelist reader.
"""
from .abi import Params, MHDError  # noqa: F401
from . import abi, ics, deck  # noqa: F401
from .solver import MHDSolver, ensemble_step, ensemble_autotune, ensemble_time  # noqa: F401
