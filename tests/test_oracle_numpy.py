"""Two independent restatements of the reference's step agree: the C++
oracle (loop per element, oracle/mhd_oracle.cpp) and the vectorised numpy
one (one array expression per Fortran statement, oracle/mhd_numpy.py), both
written from mhd3d3.f90 -- no GPU.

They share no code; exp / erfc come from different libraries (glibc; numpy and
scipy), so they agree to round-off: 1e-12 of each field's magnitude for the
fluxes and EMFs of a state, and after a few RK2 steps (measured: a few ulp).
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics
from mhd3d_mpi_fortran_gb300.abi import BC_EVEN, BC_PERIODIC, EMF_YEE, Params
from oracle.mhd_numpy import NumpyMHD
from oracle.oracle import OracleSolver

TOL = 1e-12


def close(a, b, name, scale=None):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (name, a.shape, b.shape)
    scale = max(np.abs(a).max() if scale is None else scale, 1e-300)
    err = np.abs(a - b).max() / scale
    assert err <= TOL, (name, err)


# Fields compared at the magnitude of their family: a component that is near
# zero (bz of Orszag-Tang starts at 0) carries the round-off of the others.
FAMILY = {"rho": ("rho",), "p": ("p",), "vx": ("vx", "vy", "vz"), "vy": ("vx", "vy", "vz"),
          "vz": ("vx", "vy", "vz")}
FAMILY.update({k: ("bx", "by", "bz") for k in ("bx", "by", "bz", "bi", "bj", "bk")})


def random_state(nx0, ny0, nz0, seed):
    """Positive density and pressure, random velocity and face fields: every
    limiter branch is exercised and a non-cubic grid catches axis mix-ups."""
    rng = np.random.default_rng(seed)
    s = ics.empty_state(ics.grid(nx0, ny0, nz0))
    s.rho[...] = 1.0 + 0.3 * rng.random(s.rho.shape)
    s.p[...] = 0.6 + 0.3 * rng.random(s.p.shape)
    for a in (s.vx, s.vy, s.vz):
        a[...] = 0.4 * rng.standard_normal(a.shape)
    for a in (s.bi, s.bj, s.bk):
        a[...] = 0.5 * rng.standard_normal(a.shape)
    return s


def compare_instant(prm, s):
    o = OracleSolver(prm, s)
    n = NumpyMHD(prm, s)
    for d, (fo, fn) in enumerate(zip(o.fluxes(), n.fluxes())):
        for q in range(8):
            close(fo[q], fn[q], f"flux axis {d} quantity {q}")
    for e, (eo, en) in enumerate(zip(o.emf(), n.emf())):
        close(eo, en, f"emf {e}")
    o.close()


def compare_steps(prm, s, nsteps):
    o = OracleSolver(prm, s)
    n = NumpyMHD(prm, s)
    for _ in range(nsteps):
        o.step(1)
        n.step()
    so, sn = o.fetch(), n.state()
    for k in so:
        close(so[k], sn[k], k, scale=max(np.abs(so[f]).max() for f in FAMILY[k]))
    o.close()


@pytest.mark.parametrize("recon", [1, 2, 3, 4])
def test_fluxes_and_emf_agree_on_a_random_ragged_state(recon):
    s = random_state(12, 10, 8, seed=5)
    compare_instant(Params(12, 10, 8, reconop=recon), s)


@pytest.mark.parametrize("recon", [1, 2, 3, 4])
def test_fluxes_and_emf_agree_on_orszag_tang(recon):
    s = ics.orszag_tang_3d(12, seed=2)
    compare_instant(Params(12, 12, 12, reconop=recon), s)


@pytest.mark.parametrize("recon", [1, 2, 3, 4])
@pytest.mark.parametrize("stepop", [2, 3])
def test_rk_steps_agree_on_orszag_tang(recon, stepop):
    s = ics.orszag_tang_3d(12, seed=2)
    compare_steps(Params(12, 12, 12, reconop=recon, stepop=stepop, tau=0.4 * ics.cfl_dt(s)), s, 3)


def test_the_reference_deck_agrees():
    """The scheme of mhd3d3.in (MP-WENO5, RK3, tau = 2e-4) at its 16^3 size, on
    one rank instead of the deck's 2x2x2 and with periodic halos."""
    s = ics.orszag_tang_3d(16, seed=4)
    compare_steps(Params(16, 16, 16, reconop=4, stepop=3, tau=2e-4), s, 4)


@pytest.mark.parametrize("recon", [1, 4])
def test_rk_steps_agree_on_a_random_ragged_state(recon):
    s = random_state(12, 10, 8, seed=6)
    compare_steps(Params(12, 10, 8, reconop=recon, stepop=3, tau=0.05 * ics.cfl_dt(s)), s, 2)


@pytest.mark.parametrize("recon", [1, 4])
def test_ab2_steps_agree(recon):
    """step_ab with the CFL dt; the priming step takes tau = 3e-4 as the reference
    hard-codes it (mhd3d3.f90:3356-3359)."""
    s = ics.orszag_tang_3d(12, seed=2)
    compare_steps(Params(12, 12, 12, reconop=recon, stepop=1, tau=3e-4), s, 3)


@pytest.mark.parametrize("recon,stepop", [(1, 2), (4, 3), (2, 1)])
def test_even_walls_agree(recon, stepop):
    """The wall mirror of fillx_center / fillx_face (xbc = 0, the value
    fill_hydro_mpi and fill_mag_mpi pass) on every axis, shock tube along x."""
    s = ics.shock_tube(12, axis=0, ntrans=6)
    prm = Params(12, 6, 6, reconop=recon, stepop=stepop, bc=(BC_EVEN, BC_EVEN, BC_EVEN),
                 tau=0.3 * ics.cfl_dt(s))
    compare_steps(prm, s, 3)


def test_even_walls_on_a_random_ragged_state():
    s = random_state(12, 10, 8, seed=7)
    prm = Params(12, 10, 8, reconop=1, stepop=3, bc=(BC_EVEN, BC_PERIODIC, BC_EVEN), tau=0.05 * ics.cfl_dt(s))
    compare_instant(prm, s)
    compare_steps(prm, s, 2)


@pytest.mark.parametrize("recon", [1, 2, 3, 4])
def test_yee_emf_agrees(recon):
    """get_eijk_Yee (mhd3d3.f90:1654-1752; dead code in the reference, built
    here as emf = MHD_EMF_YEE) on a random state on a ragged grid."""
    s = random_state(12, 10, 8, seed=8)
    compare_instant(Params(12, 10, 8, reconop=recon, emf=EMF_YEE), s)


@pytest.mark.parametrize("stepop", [1, 2, 3])
def test_yee_steps_agree(stepop):
    s = ics.orszag_tang_3d(12, seed=3)
    compare_steps(Params(12, 12, 12, reconop=1, stepop=stepop, emf=EMF_YEE, tau=3e-4 if stepop == 1
                         else 0.3 * ics.cfl_dt(s)), s, 3)


def test_tvd_with_the_stencil_shifts_of_mhd3d2_agrees():
    """tvd_shift = 1: the corner TVD calls honour their stencil shifts, as
    mhd3d2.f90:1137-1199 does (mhd3d3's TVD drops them)."""
    s = random_state(12, 10, 8, seed=9)
    prm = Params(12, 10, 8, reconop=2, tvd_shift=1, stepop=3, tau=0.05 * ics.cfl_dt(s))
    compare_instant(prm, s)
    compare_steps(prm, s, 2)


def test_randomised_configurations_agree():
    """Hypothesis draws the grid shape, reconstruction, stepper, halo kinds,
    EMF scheme and seed; the two restatements agree on the fluxes, the EMFs
    and two steps of every configuration it draws."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=20, deadline=None, derandomize=True)
    @hyp.given(shape=st.tuples(*[st.integers(8, 12)] * 3), recon=st.sampled_from([1, 2, 3, 4, 5]),
               stepop=st.sampled_from([1, 2, 3]), bc=st.tuples(*[st.sampled_from([0, 1, 2, 3])] * 3),
               emf=st.sampled_from([0, EMF_YEE]), seed=st.integers(0, 2 ** 16))
    def check(shape, recon, stepop, bc, emf, seed):
        s = random_state(*shape, seed=seed)
        tau = 3e-4 if stepop == 1 else 0.05 * ics.cfl_dt(s)
        prm = Params(*shape, reconop=recon, stepop=stepop, bc=bc, emf=emf, tau=tau)
        compare_instant(prm, s)
        compare_steps(prm, s, 2)

    check()


@pytest.mark.parametrize("bc", [(0, 0, 0), (1, 2, 3)])
def test_diagnostics_agree(bc):
    """N4: the oracle's compensated (Neumaier) mass and energy sums against
    exactly rounded ones; max |div B|, min rho and the CFL dt."""
    s = ics.orszag_tang_3d(12, seed=5)
    prm = Params(12, 12, 12, bc=bc, tau=0.4 * ics.cfl_dt(s))
    o, n = OracleSolver(prm, s), NumpyMHD(prm, s)
    for _ in range(2):
        o.step(1)
        n.step()
    do, dn = o.diagnostics(), n.diagnostics()
    assert do["mass"] == pytest.approx(dn["mass"], rel=1e-15, abs=0)
    assert do["energy"] == pytest.approx(dn["energy"], rel=1e-14, abs=0)
    assert abs(do["divb_max"] - dn["divb_max"]) <= 1e-13
    assert do["rho_min"] == pytest.approx(dn["rho_min"], rel=1e-14)
    assert do["dt_cfl"] == pytest.approx(dn["dt_cfl"], rel=1e-14)
    o.close()


@pytest.mark.parametrize("stepop", [2, 3])
def test_cfl_dt_mode_agrees(stepop):
    """dt_mode = CFL (no reference counterpart): RK steps take get_dt's dt."""
    s = ics.orszag_tang_3d(12, seed=6)
    compare_steps(Params(12, 12, 12, stepop=stepop, dt_mode=1, tau=1.0), s, 3)
