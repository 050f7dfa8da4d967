"""The oracle's fused mode (one pass per face / edge family, every
reconstruction evaluated where it is used) against its array passes (one
pass per Fortran statement of get_flux_stress, mhd3d3.f90:2385-2560, and
get_eijk_LFM / get_vav_center2corner, 1754-2116) -- no GPU.

Both modes call the same element functions in the same expression order, so
the states agree bit for bit after several steps of every scheme.
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics
from mhd3d_mpi_fortran_gb300.abi import (Params, BC_EVEN, BC_PERIODIC, STEP_AB2, STEP_RK2, STEP_RK3)
from oracle.oracle import OracleSolver


def run(prm, s, fused, nsteps):
    o = OracleSolver(prm, s)
    if fused:
        o.set_fused(True)
    taus = [o.step(1) for _ in range(nsteps)]
    out = o.fetch()
    flux = o.fluxes()
    emf = o.emf()
    o.close()
    return taus, out, flux, emf


def assert_same(a, b):
    taus_a, out_a, flux_a, emf_a = a
    taus_b, out_b, flux_b, emf_b = b
    assert taus_a == taus_b
    for name in out_a:
        assert np.array_equal(out_a[name], out_b[name]), name
    for fa, fb in zip(flux_a, flux_b):
        assert np.array_equal(fa, fb)
    for ea, eb in zip(emf_a, emf_b):
        assert np.array_equal(ea, eb)


@pytest.mark.parametrize("recon", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK2, STEP_RK3])
def test_fused_steps_equal_array_passes(recon, stepop):
    s = ics.orszag_tang_3d(12, seed=1)
    prm = Params(12, 12, 12, reconop=recon, stepop=stepop, tau=0.4 * ics.cfl_dt(s))
    assert_same(run(prm, s, False, 3), run(prm, s, True, 3))


@pytest.mark.parametrize("recon", [1, 2])
@pytest.mark.parametrize("tvd_shift", [0, 1])
def test_fused_walls_and_ragged_grid(recon, tvd_shift):
    """Mirror walls on x, a non-cubic grid and the TVD stencil-shift option."""
    s = ics.shock_tube(10, axis=0, ntrans=6)
    prm = Params(10, 6, 6, reconop=recon, bc=(BC_EVEN, BC_PERIODIC, BC_PERIODIC), tvd_shift=tvd_shift,
                 tau=0.3 * ics.cfl_dt(s))
    assert_same(run(prm, s, False, 2), run(prm, s, True, 2))
