"""Curvilinear (metric) mode of the oracle: consistency properties on the CPU.

The reference has no curvilinear mesh (its dxblock/dyblock/dzblock are
Cartesian, mhd3d3.f90:3473-3486), so the metric mode is specified by the
oracle and checked here by what must hold for it:
* on an identity mapping it reproduces the Cartesian scheme to round-off;
* a uniform state with B = 0 is preserved exactly on a curved mesh, and a
  uniform B converges to free-stream at second order;
* mass is conserved on a periodic mapped box and CT keeps div B at round-off;
* the cell volumes of the volume-preserving sine mapping sum to the box.
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics
from mhd3d_mpi_fortran_gb300.abi import Params, STEP_AB2, STEP_RK2, STEP_RK3, BC_OUTFLOW
from oracle.oracle import OracleSolver

SL = (slice(4, -4),) * 3


def _identity_copy(sc):
    """The Cartesian state sc on an identity-mapped grid with Phi = B.A."""
    g = sc.grid
    XI, ETA, ZETA = np.meshgrid(g.xn, g.yn, g.zn, indexing="ij")
    nodes = tuple(np.asfortranarray(a) for a in (XI, ETA, ZETA))
    sm = ics.empty_state(g, nodes)
    for k in ("rho", "vx", "vy", "vz", "p"):
        getattr(sm, k)[...] = getattr(sc, k)
    A = ics.face_areas(nodes)
    sm.bi[...] = sc.bi * A[0][..., 0]
    sm.bj[...] = sc.bj * A[1][..., 1]
    sm.bk[...] = sc.bk * A[2][..., 2]
    return sm, A


@pytest.mark.parametrize("recon,stepop", [(1, STEP_RK2), (1, STEP_AB2), (2, STEP_AB2), (5, STEP_RK3), (3, STEP_RK2)])
def test_identity_mapping_reproduces_cartesian(recon, stepop):
    sc = ics.orszag_tang_3d(12, seed=1, ny0=10, nz0=9)
    sm, A = _identity_copy(sc)
    prm = Params(12, 10, 9, reconop=recon, stepop=stepop, tau=0.5 * ics.cfl_dt(sc))
    oc, om = OracleSolver(prm, sc), OracleSolver(prm, sm)
    tc, _ = oc.step(5)
    tm, _ = om.step(5)
    fc, fm = oc.fetch(), om.fetch()
    assert tm == pytest.approx(tc, rel=1e-12)
    for k in ("rho", "vx", "vy", "vz", "p"):
        assert np.abs(fm[k] - fc[k]).max() <= 1e-12 * np.abs(fc[k]).max(), k
    bscale = max(np.abs(fc[k]).max() for k in ("bx", "by", "bz"))
    for k in ("bx", "by", "bz"):
        assert np.abs(fm[k] - fc[k]).max() <= 1e-12 * bscale, k
    for k, a, c in (("bi", A[0], 0), ("bj", A[1], 1), ("bk", A[2], 2)):
        assert np.abs(fm[k] / a[..., c] - fc[k]).max() <= 1e-12 * bscale, k


def test_uniform_flow_without_b_is_preserved_exactly():
    s = ics.uniform_flow(12, v=(0.3, -0.2, 0.1), B=(0.0, 0.0, 0.0))
    o = OracleSolver(Params(12, 12, 12, tau=2e-3), s)
    o.step(6)
    f = o.fetch()
    for k in ("rho", "vx", "vy", "vz", "p"):
        ref = getattr(s, k)[SL]
        assert np.abs(f[k][SL] - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0), k


def test_uniform_b_free_stream_converges_second_order():
    err = []
    for n in (8, 16):
        s = ics.uniform_flow(n, B=(0.3, 0.2, -0.1))
        o = OracleSolver(Params(n, n, n, tau=0.02 / n), s)
        o.step(n // 4)  # the same physical time
        err.append(float(np.abs(o.fetch()["bx"][SL] - 0.3).mean()))
    assert err[1] <= 0.3 * err[0], err


def test_mapped_orszag_tang_conserves_mass_and_div_b():
    s = ics.mapped_orszag_tang(12)
    o = OracleSolver(Params(12, 12, 12, tau=0.5 * ics.cfl_dt_mapped(s)), s)
    d0 = o.diagnostics()
    _, st = o.step(6)
    d1 = o.diagnostics()
    assert st == 0
    assert d1["mass"] == pytest.approx(d0["mass"], rel=1e-13)
    assert d0["divb_max"] <= 1e-12 and d1["divb_max"] <= 1e-12
    assert d1["energy"] < d0["energy"]  # numerical dissipation only


def test_mapped_blast_outflow_ab2_runs_clean():
    s = ics.mapped_blast(12)
    o = OracleSolver(Params(12, 12, 12, stepop=STEP_AB2, bc=(BC_OUTFLOW,) * 3, tau=0.0), s)
    tau, st = o.step(6)
    d = o.diagnostics()
    assert st == 0 and tau > 0
    assert d["divb_max"] <= 1e-12
    assert d["rho_min"] > 0.3


def test_sine_mapping_volumes_fill_the_box():
    s = ics.mapped_blast(10)
    V = OracleSolver(Params(10, 10, 10, tau=1e-3), s).volumes()
    assert V[SL].sum() == pytest.approx(1.0, abs=1e-13)
    assert V[SL].min() > 0.5 / 1000


def test_cfl_dt_mapped_matches_oracle():
    s = ics.mapped_orszag_tang(10)
    o = OracleSolver(Params(10, 10, 10, tau=1e-3), s)
    # the oracle's dt covers ghosts as get_dt does; the interior value bounds it
    assert o.diagnostics()["dt_cfl"] <= ics.cfl_dt_mapped(s) * (1 + 1e-12)
