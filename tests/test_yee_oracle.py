"""The Yee edge EMF (get_eijk_Yee, mhd3d3.f90:1654-1752; its calls are
commented out in the reference, 3354 and 3621) in the oracle -- no GPU.

Known answers the scheme implies: for a uniform state every reconstruction
returns the constant, the + and - Gaussian moments sum to (1, v), and the four
split fields of an edge add up to E = -(v x B) exactly up to rounding.  CT
keeps div B at round-off and periodic mass for any EMF, Yee included.
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics
from mhd3d_mpi_fortran_gb300.abi import Params, EMF_LFM, EMF_YEE, STEP_AB2, STEP_RK2, STEP_RK3
from oracle.oracle import OracleSolver

RECONS = [1, 2, 3, 4, 5]


def uniform_state(n=8, nord=8):
    s = ics.empty_state(ics.grid(n, n, n, nord=nord))
    s.rho[...] = 1.3
    s.p[...] = 0.7
    s.vx[...] = 0.2
    s.vy[...] = -0.1
    s.vz[...] = 0.05
    s.bi[...] = 0.3
    s.bj[...] = -0.4
    s.bk[...] = 0.25
    return s


@pytest.mark.parametrize("recon", RECONS)
def test_yee_emf_of_a_uniform_state_is_minus_v_cross_b(recon):
    s = uniform_state()
    prm = Params(8, 8, 8, reconop=recon, emf=EMF_YEE, tau=1e-3)
    ei, ej, ek = OracleSolver(prm, s).emf()
    v = np.array([0.2, -0.1, 0.05])
    b = np.array([0.3, -0.4, 0.25])
    e = -np.cross(v, b)
    for arr, ex in zip((ei, ej, ek), e):
        assert np.abs(arr - ex).max() <= 1e-14, (arr.min(), arr.max(), ex)


@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK2, STEP_RK3])
def test_yee_steps_keep_div_b_and_mass(stepop):
    s = ics.orszag_tang_3d(12, seed=3)
    prm = Params(12, 12, 12, stepop=stepop, emf=EMF_YEE, tau=0.4 * ics.cfl_dt(s))
    o = OracleSolver(prm, s)
    d0 = o.diagnostics()
    _, st = o.step(4)
    d1 = o.diagnostics()
    assert st == 0
    assert d1["divb_max"] <= 1e-12
    assert d1["mass"] == pytest.approx(d0["mass"], rel=1e-13)


def test_yee_and_lfm_converge_to_each_other():
    """Different schemes (no Alfven resistivity in Yee; Gaussian-split fields
    instead of limited corner velocities), so their EMFs differ at a finite
    resolution, but both are consistent discretisations of -(v x B): on a
    smooth noise-free state the difference shrinks at second order when the
    grid is refined."""
    diffs = []
    for n in (16, 32):
        s = ics.orszag_tang_3d(n, seed=0, amp=0.2, noise=0.0)
        e = {emf: OracleSolver(Params(n, n, n, emf=emf, tau=1e-3), s).emf() for emf in (EMF_LFM, EMF_YEE)}
        diffs.append([np.abs(a - b).max() for a, b in zip(e[EMF_LFM], e[EMF_YEE])])
    for d16, d32 in zip(*diffs):
        assert d32 > 0 and d16 / d32 >= 2.8, (d16, d32)
