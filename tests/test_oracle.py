"""CPU tests of the oracle (the C++ FP64 restatement) -- no GPU.

The reference ships no tests or golden vectors; these pin the restatement
with the invariants its own artefacts imply: point symmetry of Orszag-Tang
(process_mhd_2d.m:95-102), axis permutation of the shock tube
(mhd3d3.f90:3523-3569), div B from CT (mhd3d3.f90:3909-3933), periodic mass
conservation, plus known answers of the reconstructions.
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics
from mhd3d_mpi_fortran_gb300.abi import (Params, BC_PERIODIC, BC_EVEN, BC_REFLECT, BC_OUTFLOW,
                                         STEP_AB2, STEP_RK2, STEP_RK3, ST_NAN, ST_NEG_RHO)
from oracle.oracle import OracleSolver, recon_line

RECONS = [1, 2, 3, 4, 5]


def interior(a, ng, extra=(0, 0, 0)):
    return a[ng:a.shape[0] - ng + 0, ng:a.shape[1] - ng, ng:a.shape[2] - ng]


def prm_for(s, **kw):
    g = s.grid
    kw.setdefault("tau", 0.5 * ics.cfl_dt(s))
    return Params(g.nx0, g.ny0, g.nz0, nord=2 * g.ng, **kw)


@pytest.mark.parametrize("recon", RECONS)
@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK2, STEP_RK3])
def test_uniform_state_stays_uniform(recon, stepop):
    g = ics.grid(8, 8, 8)
    s = ics.empty_state(g)
    s.rho[...] = 1.3
    s.p[...] = 0.7
    s.vx[...] = 0.2
    s.vy[...] = -0.1
    s.vz[...] = 0.05
    s.bi[...] = 0.3
    s.bj[...] = -0.2
    s.bk[...] = 0.1
    o = OracleSolver(Params(8, 8, 8, reconop=recon, stepop=stepop, tau=1e-3), s)
    o.step(3)
    f = o.fetch()
    for k, v in (("rho", 1.3), ("p", 0.7), ("vx", 0.2), ("vy", -0.1), ("vz", 0.05)):
        assert np.allclose(f[k], v, rtol=1e-13, atol=1e-14), k
    assert np.allclose(f["bi"], 0.3, rtol=0, atol=1e-15)


@pytest.mark.parametrize("recon", RECONS)
def test_periodic_mass_conservation_and_divb(recon):
    s = ics.orszag_tang_3d(16, seed=1)
    o = OracleSolver(prm_for(s, reconop=recon), s)
    d0 = o.diagnostics()
    o.step(4)
    d1 = o.diagnostics()
    assert abs(d1["mass"] - d0["mass"]) <= 1e-13 * d0["mass"]
    assert d0["divb_max"] <= 1e-12
    assert d1["divb_max"] <= 1e-12


def test_turbulence_divb_and_mass():
    s = ics.turbulence(16, seed=3)
    o = OracleSolver(prm_for(s), s)
    d0 = o.diagnostics()
    assert d0["divb_max"] <= 1e-12
    o.step(3)
    d1 = o.diagnostics()
    assert d1["divb_max"] <= 1e-12
    assert abs(d1["mass"] - d0["mass"]) <= 1e-13 * d0["mass"]


@pytest.mark.parametrize("recon", [1, 2, 4])
def test_shock_tube_axis_permutation(recon):
    """x, y and z tubes (mhd3d3.f90:3531-3569) give identical profiles."""
    n, nt = 32, 8
    prof = []
    for axis in (0, 1, 2):
        s = ics.shock_tube(n, axis=axis, ntrans=nt)
        prm = Params(*(n if a == axis else nt for a in range(3)), reconop=recon, tau=2e-3,
                     bc=(BC_EVEN, BC_EVEN, BC_EVEN))
        o = OracleSolver(prm, s)
        o.step(20)
        f = o.fetch()
        sl = [4] * 3
        sl[axis] = slice(None)
        normal_v = ("vx", "vy", "vz")[axis]
        trans_b = ("bx", "by", "bz")[(axis + 1) % 3]
        prof.append(np.stack([f["rho"][tuple(sl)], f["p"][tuple(sl)], f[normal_v][tuple(sl)],
                              f[trans_b][tuple(sl)]]))
    assert np.array_equal(prof[0], prof[1])
    assert np.array_equal(prof[1], prof[2])
    # the tube evolved
    assert np.ptp(prof[2][0]) > 0.5


def test_orszag_tang_point_symmetry():
    """process_mhd_2d.m:95-102: var(i,j) - var(n+1-i, n+1-j) stays at round-off."""
    n = 32
    s = ics.orszag_tang_2d(n, nz0=8)
    prm = Params(n, n, 8, tau=0.5 * ics.cfl_dt(s))
    o = OracleSolver(prm, s)
    o.step(30)
    f = o.fetch()
    ng = 4
    r = f["rho"][ng:ng + n, ng:ng + n, ng]
    p = f["p"][ng:ng + n, ng:ng + n, ng]
    sym = lambda a: a[::-1, ::-1]
    scale = np.abs(r).max()
    assert np.abs(r - sym(r)).max() <= 1e-10 * scale
    assert np.abs(p - sym(p)).max() <= 1e-10 * np.abs(p).max()
    assert np.ptp(r) > 0.01  # the vortex evolved


@pytest.mark.parametrize("kind", [BC_PERIODIC, BC_EVEN, BC_REFLECT, BC_OUTFLOW])
def test_fill_maps(kind):
    """Ghost values after init equal the per-axis images of fill_*_mpi."""
    g = ics.grid(6, 5, 7)
    rng = np.random.default_rng(5)
    s = ics.empty_state(g)
    for a in s.arrays():
        a[...] = rng.uniform(0.5, 1.5, size=a.shape)
    o = OracleSolver(Params(6, 5, 7, bc=(kind,) * 3, tau=1e-3), s)
    f = o.fetch()
    ng = 4

    def src(x, n0, face):
        hi = ng + n0 if face else ng + n0 - 1
        if ng <= x <= hi:
            return x, 1.0
        lo = x < ng
        if kind == BC_PERIODIC:
            return (x + n0 if lo else x - n0), 1.0
        if kind == BC_OUTFLOW:
            return (ng if lo else hi), 1.0
        if not face:
            return (2 * ng - 1 - x if lo else 2 * n0 + 2 * ng - 1 - x), -1.0
        return (2 * ng - x if lo else 2 * n0 + 2 * ng - x), -1.0

    n0 = (6, 5, 7)
    for name, fa, var in (("rho", -1, 0), ("vx", -1, 1), ("vy", -1, 2), ("bi", 0, 0), ("bj", 1, 0), ("bk", 2, 0)):
        orig = getattr(s, name)
        got = f[name]
        for idx in np.ndindex(*orig.shape):
            sidx, sgn = [], 1.0
            for ax in range(3):
                x, fl = src(idx[ax], n0[ax], fa == ax)
                sidx.append(x)
                if fl < 0 and kind == BC_REFLECT and var == ax + 1 and x != idx[ax]:
                    sgn = -sgn
            assert got[idx] == sgn * orig[tuple(sidx)], (name, idx)


def test_recon_pdm_linear_exact():
    prm = Params(8, 8, 8, reconop=1)
    f = 0.3 + 0.25 * np.arange(20.0)
    fl, fr = recon_line(prm, f)
    for c in range(4, 12):
        face = 0.5 * (f[c - 1] + f[c])
        assert fl[c] == pytest.approx(face, abs=1e-14)
        assert fr[c] == pytest.approx(face, abs=1e-14)


@pytest.mark.parametrize("recon", RECONS)
def test_recon_monotone_on_step(recon):
    prm = Params(8, 8, 8, reconop=recon)
    f = np.where(np.arange(24) < 12, 1.0, 0.125)
    fl, fr = recon_line(prm, f)
    for c in range(4, 16):
        lo, hi = min(f[c - 1], f[c]), max(f[c - 1], f[c])
        if recon in (1, 2, 4, 5):  # limited schemes stay within the neighbours
            assert lo - 1e-12 <= fl[c] <= hi + 1e-12
            assert lo - 1e-12 <= fr[c] <= hi + 1e-12


def test_recon_weno_order():
    """WENO5 face values converge at high order on smooth data."""
    errs = []
    for n in (32, 64):
        x = (np.arange(n + 8) - 4 + 0.5) / n
        cell = (np.cos(2 * np.pi * (x - 0.5 / n)) - np.cos(2 * np.pi * (x + 0.5 / n))) / (2 * np.pi / n)  # cell means of sin
        prm = Params(8, 8, 8, reconop=3, eps=1e-40)
        fl, fr = recon_line(prm, cell)
        faces = np.sin(2 * np.pi * (np.arange(n + 8) - 4) / n)
        errs.append(np.abs(fl[4:n + 4] - faces[4:n + 4]).max())
    assert errs[0] / errs[1] > 16.0  # at least 4th order observed


def test_status_bits_on_poisoned_state():
    s = ics.orszag_tang_3d(8)
    s.rho[6, 6, 6] = np.nan
    o = OracleSolver(prm_for(ics.orszag_tang_3d(8)), s)
    _, st = o.step(1)
    assert st & ST_NAN
    s = ics.orszag_tang_3d(8)
    s.rho[6, 6, 6] = -1.0
    o = OracleSolver(prm_for(ics.orszag_tang_3d(8)), s)
    _, st = o.step(1)
    assert st & ST_NEG_RHO
