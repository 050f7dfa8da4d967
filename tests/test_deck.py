"""Namelist deck reader (read_input, mhd3d3.f90:147-197) and IC generators."""
import numpy as np

from mhd3d_mpi_fortran_gb300 import deck, ics
from mhd3d_mpi_fortran_gb300.abi import BC_PERIODIC

DECK = """ &dom
 xmin=0., xmax=2., ymin=-1., ymax=1., zmin=0., zmax=1.
/

 &grid
 nx0G=32, ny0G=24, nz0G=16, xprocs=1, yprocs=1, zprocs=1
/

 &comset
 nord=6, reconop=4, stepop=3, outop=2
/

 &list
 nts=5, tau=1.5e-4, nframes=3, nrst=0, nfdump=10
/

 &free
 cfl=.25, pdmb=4., eps=1.d-8, alpha=2., beta=4.
/
"""


def test_read_deck_groups_and_values():
    d = deck.read_deck(DECK)
    assert d["grid"]["nx0g"] == 32 and d["grid"]["nz0g"] == 16
    assert d["comset"]["reconop"] == 4
    assert d["list"]["tau"] == 1.5e-4
    assert d["free"]["cfl"] == 0.25 and d["free"]["eps"] == 1e-8
    p = deck.params_from_deck(d, bc=BC_PERIODIC)
    assert (p.nx0, p.ny0, p.nz0, p.nord, p.reconop, p.stepop) == (32, 24, 16, 6, 4, 3)
    assert p.tau == 1.5e-4 and p.cfl == 0.25 and p.bc == (0, 0, 0)
    lo, hi = deck.domain_from_deck(d)
    assert lo == (0.0, -1.0, 0.0) and hi == (2.0, 1.0, 1.0)


def test_grid_matches_init_geom():
    g = ics.grid(16, 8, 4, nord=8, lo=(-1, -1, -1), hi=(1, 1, 1))
    assert g.xn.shape == (16 + 8 + 1,)
    assert np.allclose(g.dx, 2.0 / 16)
    assert g.xn[4] == -1.0 and g.xn[4 + 16] == 1.0
    # ghost nodes extended linearly (mhd3d3.f90:3418-3426)
    assert np.isclose(g.xn[0], -1.0 - 4 * 2.0 / 16)


def test_ot3d_is_divergence_free():
    s = ics.orszag_tang_3d(16)
    g = s.grid
    ng = g.ng
    sl = slice(ng, ng + 16)
    div = (np.diff(s.bi, axis=0)[sl, sl, sl] / g.dx[ng] + np.diff(s.bj, axis=1)[sl, sl, sl] / g.dy[ng] +
           np.diff(s.bk, axis=2)[sl, sl, sl] / g.dz[ng])
    assert np.abs(div).max() < 1e-12
    assert abs(s.rho[sl, sl, sl].mean() - 25 / (36 * np.pi)) < 1e-3


def test_turbulence_rms_and_divergence():
    s = ics.turbulence(16, seed=2)
    g = s.grid
    ng = g.ng
    sl = slice(ng, ng + 16)
    v2 = s.vx[sl, sl, sl] ** 2 + s.vy[sl, sl, sl] ** 2 + s.vz[sl, sl, sl] ** 2
    assert abs(np.sqrt(v2.mean()) - 1.0) < 1e-12
    div = (np.diff(s.bi, axis=0)[sl, sl, sl] + np.diff(s.bj, axis=1)[sl, sl, sl] +
           np.diff(s.bk, axis=2)[sl, sl, sl]) / g.dx[ng]
    assert np.abs(div).max() < 1e-12


def test_blast_bws_is_the_reference_cylinder():
    """init_ic_bws (mhd3d2.f90:3358-3418): p = 10 inside xc^2 + yc^2 < .01, .1
    outside, whatever z; rho = 1, v = 0, bi = bj = .5, bk = 0."""
    s = ics.blast_bws(32, nz0=4, lo=(-0.5, -0.5, 0.0), hi=(0.5, 0.5, 1.0))
    xc, yc, zc = s.grid.centres()
    inside = (xc[:, None] ** 2 + yc[None, :] ** 2) < 0.01
    assert inside.any() and (~inside).any()
    for k in range(s.p.shape[2]):
        assert np.array_equal(s.p[:, :, k], np.where(inside, 10.0, 0.1))
    assert np.all(s.rho == 1.0) and np.all(s.vx == 0) and np.all(s.vy == 0) and np.all(s.vz == 0)
    assert np.all(s.bi == 0.5) and np.all(s.bj == 0.5) and np.all(s.bk == 0.0)


def test_blast_bws_runs_in_the_oracle():
    """The cylinder centred in a periodic box: clean steps, div B at round-off,
    mass conserved."""
    import pytest
    from mhd3d_mpi_fortran_gb300.abi import Params
    from oracle.oracle import OracleSolver
    s = ics.blast_bws(16, nz0=4, lo=(-0.5, -0.5, 0.0), hi=(0.5, 0.5, 1.0))
    o = OracleSolver(Params(16, 16, 4, tau=0.3 * ics.cfl_dt(s)), s)
    d0 = o.diagnostics()
    _, st = o.step(3)
    d1 = o.diagnostics()
    assert st == 0
    assert d1["divb_max"] <= 1e-12
    assert d1["mass"] == pytest.approx(d0["mass"], rel=1e-13)
