"""GPU parity over long horizons and at the reference decks' other settings.

Every case runs the CUDA path through the C ABI and compares it with the FP64
oracle on the same inputs:

* 3 ghost layers (nord = 6), the ghost depth of mhd3d2.in (``nord=6,
  reconop=4, stepop=3``, mhd3d2.in:10) with mhd3d2's 2-D setting: periodic x
  and y (mhd3d2.f90:3063-3064) and the z-constant fill (fillz_even1,
  mhd3d2.f90:687-697, 731-772), for every reconstruction that runs with 3
  ghosts and every stepper; the FP32 column sweeps at that depth too;
* 100 steps of the default deck's scheme, MP-WENO5 + RK3 (mhd3d3.in:10;
  step_rk3 mhd3d3.f90:3715-3792, MPWENO5 1405-1596);
* 100 AB2 steps (step_ab, mhd3d3.f90:3602-3644) of a blast between walls and
  with outflow boundaries, including the sequence of CFL time steps;
* the FP32 production path against the all-FP64 mode on the benchmark's own
  workload (decaying turbulence, PDM + RK2) at 128^3 over 100 steps.
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics, MHDSolver
from mhd3d_mpi_fortran_gb300.abi import (Params, BC_PERIODIC, BC_OUTFLOW, BC_REFLECT, BC_EVEN, STEP_AB2,
                                         STEP_RK2, STEP_RK3, FP32, FP64)
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "bi", "bj", "bk")
BC2D = (BC_PERIODIC, BC_PERIODIC, BC_OUTFLOW)


def rel_l2(a, b):
    return np.sqrt(np.sum((a - b) ** 2)) / max(np.sqrt(np.sum(b ** 2)), 1e-300)


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def interior(a, ng):
    return a[ng:a.shape[0] - ng, ng:a.shape[1] - ng, ng:a.shape[2] - ng]


@pytest.mark.parametrize("recon", [2, 3, 4, 5])
@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK2, STEP_RK3])
def test_nord6_steps_fp64_match_oracle(recon, stepop):
    """Three ghost layers: TVD, WENO5, MP-WENO5 and TVD-MC with every stepper
    on the 2-D Orszag-Tang vortex (init_ic_otv, mhd3d2.f90:3420-3438) over
    x-y periodic / z-constant halos; 4 steps, every array incl. ghosts."""
    s = ics.orszag_tang_2d(12, nz0=8, nord=6)
    prm = Params(12, 12, 8, nord=6, reconop=recon, stepop=stepop, bc=BC2D,
                 tau=0.5 * ics.cfl_dt(s) if stepop != STEP_AB2 else 1e-4)
    with MHDSolver(prm, s) as gpu:
        tg, sg = gpu.step(4)
        fg = gpu.fetch()
    o = OracleSolver(prm, s)
    to, so = o.step(4)
    fo = o.fetch()
    assert tg == pytest.approx(to, rel=1e-13)
    assert sg == so
    for k in FIELDS:
        assert relmax(fg[k], fo[k]) <= 1e-11, k


def test_nord6_mhd3d2_deck_fp64_and_fp32():
    """mhd3d2.in's scheme at its ghost depth: MP-WENO5 + RK3, nord = 6, tau =
    1e-4 (mhd3d2.in:10, 14) from init_ic_otv on a 32^2 x 8 grid, 40 steps.
    FP64 matches the oracle (relative L2 <= 1e-10 per field) and stays exactly
    z-invariant; the FP32 path (column sweeps, whose register window reaches
    4 cells and is clamped to the 3-layer halo) stays within 1e-5 relative L1
    of FP64, z-invariant, and bit-identical to the FP32 face tiles."""
    s = ics.orszag_tang_2d(32, nz0=8, nord=6)
    prm = Params(32, 32, 8, nord=6, reconop=4, stepop=STEP_RK3, bc=BC2D, tau=1e-4)
    with MHDSolver(prm, s) as gpu:
        _, st = gpu.step(40)
        f64 = gpu.fetch()
    assert st == 0
    o = OracleSolver(prm, s)
    o.step(40)
    fo = o.fetch()
    for k in FIELDS:
        assert rel_l2(f64[k], fo[k]) <= 1e-10, k
    p32 = Params(32, 32, 8, nord=6, reconop=4, stepop=STEP_RK3, bc=BC2D, tau=1e-4, precision=FP32)
    res = {}
    for td in (32, 8):
        with MHDSolver(p32, s) as gpu:
            gpu.set_tiles(td, 8)
            gpu.step(40)
            res[td] = gpu.fetch()
    for k in FIELDS:
        assert np.array_equal(res[32][k], res[8][k]), k
    f32 = res[32]
    for k in ("rho", "p", "vx", "vy", "bi", "bj"):
        a, b = interior(f32[k], 3), interior(f64[k], 3)
        assert np.abs(a - b).sum() / np.abs(b).sum() <= 1e-5, k
        for z in range(1, a.shape[2]):
            assert np.array_equal(a[:, :, z], a[:, :, 0]), (k, z)
            assert np.array_equal(interior(f64[k], 3)[:, :, z], b[:, :, 0]), (k, z)


@pytest.mark.slow
def test_mpweno_rk3_100_steps_32cubed():
    """The default deck's scheme (MP-WENO5 + RK3, mhd3d3.in:10) over 100 steps
    of the 3-D Orszag-Tang problem at 32^3, fixed tau = the CFL-0.3 dt of the
    initial state: relative L2 <= 1e-10 per field, div B <= 1e-12."""
    s = ics.orszag_tang_3d(32, seed=0)
    prm = Params(32, 32, 32, reconop=4, stepop=STEP_RK3, cfl=0.3, tau=ics.cfl_dt(s, cfl=0.3))
    with MHDSolver(prm, s) as gpu:
        tg, sg = gpu.step(100)
        fg = gpu.fetch()
        dg = gpu.diagnostics()
    o = OracleSolver(prm, s)
    to, so = o.step(100)
    fo = o.fetch()
    assert tg == to and sg == so
    for k in FIELDS:
        assert rel_l2(fg[k], fo[k]) <= 1e-10, k
    assert dg["divb_max"] <= 1e-12


@pytest.mark.slow
@pytest.mark.parametrize("bc", [BC_OUTFLOW, BC_REFLECT, BC_EVEN])
def test_ab2_blast_100_steps_with_cfl_dt_sequence(bc):
    """100 AB2 steps of the magnetised blast at 24^3 between walls (even and
    reflecting mirrors) and with outflow boundaries.  Each step takes the CFL
    dt of its own input (get_dt in step_ab, mhd3d3.f90:3609) and feeds
    tau/tau0 to the next predictor (advance_predictor_ab, 3821-3840), so a
    slip compounds over the run: every step's dt matches the oracle's to
    1e-12 relative, and the final state to relative L2 <= 1e-10."""
    s = ics.blast(24)
    prm = Params(24, 24, 24, reconop=1, stepop=STEP_AB2, bc=(bc,) * 3, tau=3e-4)
    o = OracleSolver(prm, s)
    with MHDSolver(prm, s) as gpu:
        for n in range(100):
            tg, sg = gpu.step(1)
            to, so = o.step(1)
            assert tg == pytest.approx(to, rel=1e-12), n
            assert sg == so == 0, n
        fg = gpu.fetch()
        dg = gpu.diagnostics()
    fo = o.fetch()
    for k in FIELDS:
        assert rel_l2(fg[k], fo[k]) <= 1e-10, k
    assert dg["divb_max"] <= 1e-12


@pytest.mark.slow
def test_fp32_budget_on_the_bench_workload_128cubed():
    """The production FP32 path on the benchmark's workload (seeded solenoidal
    turbulence, E(k) ~ k^-2 on 2 <= k <= 8, PDM + RK2, the bench's dt = 0.8 x
    the initial CFL-0.3 dt) at 128^3 over 100 steps, against the all-FP64 mode
    on the same inputs: relative L1 <= 1e-5 per field, FP32 div B at FP32
    round-off of the face field (max |div B| dx / max |B| <= 1e-5), and mass
    conserved to FP32 round-off."""
    s = ics.turbulence(128, seed=0)
    tau = 0.8 * ics.cfl_dt(s, cfl=0.3)
    out, diag = {}, {}
    for prec in (FP64, FP32):
        with MHDSolver(Params(128, 128, 128, reconop=1, stepop=STEP_RK2, precision=prec, tau=tau), s) as g:
            d0 = g.diagnostics()
            _, st = g.step(100)
            assert st == 0
            out[prec] = g.fetch()
            diag[prec] = (d0, g.diagnostics())
    for k in ("rho", "vx", "vy", "vz", "p", "bi", "bj", "bk"):
        a, b = interior(out[FP32][k], 4), interior(out[FP64][k], 4)
        l1 = np.abs(a - b).sum() / np.abs(b).sum()
        assert l1 <= 1e-5, (k, l1)
    d0, d1 = diag[FP32]
    # max |div B| in units of max|B| / dx: a few FP32 ulps of the face field
    bmax = max(np.abs(out[FP32][k]).max() for k in ("bi", "bj", "bk"))
    assert d1["divb_max"] * (1.0 / 128) / bmax <= 1e-5
    assert abs(d1["mass"] - d0["mass"]) <= 1e-5 * d0["mass"]
    d0, d1 = diag[FP64]
    assert d1["divb_max"] <= 1e-12
    assert abs(d1["mass"] - d0["mass"]) <= 1e-13 * d0["mass"]
