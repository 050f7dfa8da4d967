"""GPU parity: libmhdgpu.so (through the C ABI) against the CPU oracle.

FP64 mode follows the reference's expression order with no FMA, so kernel
outputs agree with the oracle to a few ulps (only exp/erfc differ: CUDA vs
glibc).  Tolerances are written per test.  FP32 mode is checked against the
FP64 solution with an error budget, as the production path.
"""
import ctypes as C

import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics, MHDSolver, ensemble_step
from mhd3d_mpi_fortran_gb300.abi import (Params, BC_PERIODIC, BC_EVEN, BC_REFLECT, BC_OUTFLOW,
                                         STEP_AB2, STEP_RK2, STEP_RK3, FP32, FP64, ST_NAN, ST_NEG_RHO,
                                         ST_TIMEOUT, E_OK, E_ARG, E_TIMEOUT, DT_CFL)
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

RECONS = [1, 2, 3, 4, 5]
FIELDS = ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "bi", "bj", "bk")


def rand_state(nx0, ny0, nz0, seed=0, nord=8):
    """Smooth waves plus a density/pressure jump and random face B."""
    g = ics.grid(nx0, ny0, nz0, nord=nord)
    s = ics.empty_state(g)
    rng = np.random.default_rng(seed)
    xc, yc, zc = [c.reshape(sh) for c, sh in zip(g.centres(), ((-1, 1, 1), (1, -1, 1), (1, 1, -1)))]
    s.rho[...] = 1.0 + 0.3 * np.sin(2 * np.pi * xc) * np.cos(2 * np.pi * yc) + 0.5 * (zc > 0.5)
    s.p[...] = 0.8 + 0.2 * np.cos(2 * np.pi * (xc + zc)) + 0.4 * (xc > 0.6)
    s.vx[...] = 0.4 * np.sin(2 * np.pi * yc) + 0.05 * rng.standard_normal(s.vx.shape)
    s.vy[...] = -0.3 * np.sin(2 * np.pi * zc) + 0.05 * rng.standard_normal(s.vy.shape)
    s.vz[...] = 0.2 * np.cos(2 * np.pi * xc) + 0.05 * rng.standard_normal(s.vz.shape)
    for a in (s.bi, s.bj, s.bk):
        a[...] = 0.3 * rng.standard_normal(a.shape)
    return s


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def rel_l2(a, b):
    return np.sqrt(np.sum((a - b) ** 2)) / max(np.sqrt(np.sum(b ** 2)), 1e-300)


@pytest.mark.parametrize("recon", RECONS)
def test_fluxes_fp64_match_oracle(recon):
    s = rand_state(12, 10, 9, seed=recon)
    prm = Params(12, 10, 9, reconop=recon, tau=1e-3)
    with MHDSolver(prm, s) as gpu:
        fg = gpu.debug_fluxes()
    fo = OracleSolver(prm, s).fluxes()
    for d in range(3):
        for q in range(8):
            assert relmax(fg[d][q], fo[d][q]) <= 1e-13, (d, q)


@pytest.mark.parametrize("recon", RECONS)
@pytest.mark.parametrize("shift", [0, 1])
def test_emf_fp64_match_oracle(recon, shift):
    if shift and recon not in (2, 5):
        pytest.skip("stencil shifts only differ for TVD")
    s = rand_state(11, 12, 10, seed=10 + recon)
    prm = Params(11, 12, 10, reconop=recon, tvd_shift=shift, tau=1e-3)
    with MHDSolver(prm, s) as gpu:
        eg = gpu.debug_emf()
    eo = OracleSolver(prm, s).emf()
    for e in range(3):
        assert relmax(eg[e], eo[e]) <= 1e-13, e


@pytest.mark.parametrize("recon", [1, 3, 4])
@pytest.mark.parametrize("shape", [(32, 8, 16), (64, 17, 9), (33, 16, 8)])
def test_emf_multi_tile_fp64(shape, recon):
    """Shared-memory EMF tiles over several blocks per axis.  PDM ej / ek: a
    transverse axis with n0 + 1 = 32 q + 1 (x) or 8 q + 1 (the other
    transverse axis) edges ends in a tile one edge wider instead of a block
    holding one edge row.  WENO5 / MP-WENO5: row and column reconstructions
    shared through shared memory.  Every edge matches the oracle."""
    s = rand_state(*shape, seed=sum(shape))
    prm = Params(*shape, reconop=recon, tau=1e-3)
    with MHDSolver(prm, s) as gpu:
        eg = gpu.debug_emf()
    eo = OracleSolver(prm, s).emf()
    for e in range(3):
        assert relmax(eg[e], eo[e]) <= 1e-13, e


@pytest.mark.parametrize("recon", RECONS)
@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK2, STEP_RK3])
def test_steps_fp64_match_oracle(recon, stepop):
    s = ics.orszag_tang_3d(12, seed=recon, ny0=10, nz0=9)
    prm = Params(12, 10, 9, reconop=recon, stepop=stepop, tau=0.5 * ics.cfl_dt(s),
                 nord=8)
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


@pytest.mark.parametrize("kind", [BC_EVEN, BC_REFLECT, BC_OUTFLOW])
def test_boundary_kinds_fp64(kind):
    s = ics.blast(12)
    prm = Params(12, 12, 12, bc=(kind,) * 3, tau=0.5 * ics.cfl_dt(s))
    with MHDSolver(prm, s) as gpu:
        gpu.step(5)
        fg = gpu.fetch()
    o = OracleSolver(prm, s)
    o.step(5)
    fo = o.fetch()
    for k in FIELDS:
        assert relmax(fg[k], fo[k]) <= 1e-11, k


def test_cfl_dt_mode_and_diagnostics():
    s = ics.turbulence(16, seed=4)
    prm = Params(16, 16, 16, dt_mode=DT_CFL, tau=1.0)
    with MHDSolver(prm, s) as gpu:
        dg0 = gpu.diagnostics()
        tg, _ = gpu.step(3)
        dg = gpu.diagnostics()
    o = OracleSolver(prm, s)
    do0 = o.diagnostics()
    to, _ = o.step(3)
    do = o.diagnostics()
    assert dg0["dt_cfl"] == pytest.approx(do0["dt_cfl"], rel=1e-14)
    assert tg == pytest.approx(to, rel=1e-12)
    assert dg["mass"] == pytest.approx(do["mass"], rel=1e-13)
    assert dg["energy"] == pytest.approx(do["energy"], rel=1e-12)
    assert dg["divb_max"] <= 1e-12 and do["divb_max"] <= 1e-12
    assert dg["rho_min"] == pytest.approx(do["rho_min"], rel=1e-12)


@pytest.mark.parametrize("stepop", [STEP_RK2, STEP_RK3])
def test_cfl_dt_sequence_across_graphs_diagnostics_and_batched_steps(stepop):
    """Cartesian RK steps take the CFL dt that the previous step's last stage
    accumulated for their starting state, and the first stage stores U^n;
    the first step, a step after a batched ensemble step (which runs its own
    CFL pass) and graph replays recompute or reuse it.  Every step's CFL dt
    (dt_mode = CFL) and the final fields match the oracle stepped alongside."""
    s = ics.turbulence(16, seed=11)
    prm = Params(16, 16, 16, stepop=stepop, dt_mode=DT_CFL, tau=1.0)
    o = OracleSolver(prm, s)
    with MHDSolver(prm, s) as gpu:
        seq = []
        for n in range(3):
            tg, sg = gpu.step(1)
            to, so = o.step(1)
            seq.append((tg, to))
            assert sg == so == 0
        gpu.diagnostics()  # a peek at the CFL dt between steps leaves the pending one alone
        tg, _ = gpu.step(2, graph=True)
        to, _ = o.step(2)
        seq.append((tg, to))
        ensemble_step([gpu], 1)
        o.step(1)
        tg, _ = gpu.step(1)
        to, _ = o.step(1)
        seq.append((tg, to))
        tg, _ = gpu.step(2, graph=True)
        to, _ = o.step(2)
        seq.append((tg, to))
        fg = gpu.fetch()
    fo = o.fetch()
    for tg, to in seq:
        assert tg == pytest.approx(to, rel=1e-12)
    for k in FIELDS:
        assert relmax(fg[k], fo[k]) <= 1e-11, k


@pytest.mark.slow
def test_whole_step_parity_64cubed_100_steps():
    """All-FP64 mode vs the oracle: 64^3 periodic 3-D Orszag-Tang, PDM + RK2,
    fixed tau = the CFL-0.3 dt of the initial state, 100 steps: relative L2
    <= 1e-10 per field and div B <= 1e-12."""
    s = ics.orszag_tang_3d(64, seed=0)
    prm = Params(64, 64, 64, reconop=1, stepop=STEP_RK2, cfl=0.3, tau=ics.cfl_dt(s, cfl=0.3))
    with MHDSolver(prm, s) as gpu:
        gpu.step(100)
        fg = gpu.fetch()
        dg = gpu.diagnostics()
    o = OracleSolver(prm, s)
    o.step(100)
    fo = o.fetch()
    for k in FIELDS:
        assert rel_l2(fg[k], fo[k]) <= 1e-10, k
    assert dg["divb_max"] <= 1e-12


@pytest.mark.parametrize("recon", RECONS)
def test_fp32_error_budget_vs_fp64(recon):
    """FP32 production path (fast reciprocal quotients, fitted erfc) against
    the all-FP64 mode for every reconstruction."""
    s = ics.orszag_tang_3d(32, seed=0)
    tau = ics.cfl_dt(s)
    res = {}
    for prec in (FP64, FP32):
        with MHDSolver(Params(32, 32, 32, reconop=recon, precision=prec, tau=tau), s) as gpu:
            gpu.step(20)
            res[prec] = gpu.fetch()
            if prec == FP32:
                d32 = gpu.diagnostics()
    for k in ("rho", "p", "vx", "bi"):
        a, b = res[FP32][k], res[FP64][k]
        l1 = np.abs(a - b).sum() / np.abs(b).sum()
        assert l1 <= 1e-5, (k, l1)
    # CT keeps div B at FP32 round-off
    assert d32["divb_max"] <= 1e-4


def test_graph_replay_equals_stream_fp64():
    s = ics.orszag_tang_3d(16, seed=2)
    prm = Params(16, 16, 16, tau=0.5 * ics.cfl_dt(s))
    with MHDSolver(prm, s) as a, MHDSolver(prm, s) as b:
        a.step(6)
        b.step(3, graph=True)
        b.step(3, graph=True)
        fa, fb = a.fetch(), b.fetch()
    for k in FIELDS:
        assert np.array_equal(fa[k], fb[k]), k


def test_ensemble_equals_sequential_fp64():
    sizes = (12, 16, 8)
    states = [ics.orszag_tang_3d(n, seed=i, amp=0.5 + 0.25 * i) for i, n in enumerate(sizes)]
    prms = [Params(n, n, n, tau=0.5 * ics.cfl_dt(st)) for n, st in zip(sizes, states)]
    seq = []
    for prm, st in zip(prms, states):
        with MHDSolver(prm, st) as g:
            g.step(3)
            seq.append(g.fetch())
    ens = [MHDSolver(p, st) for p, st in zip(prms, states)]
    ensemble_step(ens, 3)
    for e, ref in zip(ens, seq):
        got = e.fetch()
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), k
        e.close()


@pytest.mark.parametrize("prec", [FP64, FP32])
def test_status_bits_from_poisoned_input(prec):
    base = ics.orszag_tang_3d(8)
    tau = 0.5 * ics.cfl_dt(base)
    s = ics.orszag_tang_3d(8)
    s.rho[6, 6, 6] = np.nan
    with MHDSolver(Params(8, 8, 8, precision=prec, tau=tau), s) as g:
        _, st = g.step(1)
    assert st & ST_NAN
    s = ics.orszag_tang_3d(8)
    s.rho[6, 6, 6] = -1.0
    with MHDSolver(Params(8, 8, 8, precision=prec, tau=tau), s) as g:
        _, st = g.step(1)
    assert st & ST_NEG_RHO


def test_wait_bound_timeout_leaves_the_handle_usable():
    """A host wait that runs out (mhd_set_wait_bound) returns MHD_E_TIMEOUT with
    MHD_ST_TIMEOUT while the enqueued steps keep running; with the bound
    restored the next call waits for them, and the state equals an
    uninterrupted run.  Nothing on the device faults or hangs: the steps are
    ordinary FP64 steps (about 0.2 s of device time) that finish by themselves."""
    s = ics.orszag_tang_3d(96, seed=1)
    prm = Params(96, 96, 96, precision=FP64, tau=0.3 * ics.cfl_dt(s))
    with MHDSolver(prm, s) as g, MHDSolver(prm, s) as ref:
        lib = g.lib
        tau, st = C.c_double(), C.c_uint32()
        assert lib.mhd_set_wait_bound(1e-4) == E_OK
        try:
            rc = lib.mhd_step_n(g.h, 20, C.byref(tau), C.byref(st))
        finally:
            assert lib.mhd_set_wait_bound(600.0) == E_OK
        assert rc == E_TIMEOUT, rc
        assert st.value & ST_TIMEOUT
        assert b"wait bound" in lib.mhd_last_error()
        g.step(1)  # waits for the 20 steps in flight, then one more
        ref.step(21)
        got, want = g.fetch(), ref.fetch()
        for k in FIELDS:
            assert np.array_equal(got[k], want[k]), k
    assert lib.mhd_set_wait_bound(0.0) == E_ARG


@pytest.mark.parametrize("prec,stepop", [(FP64, STEP_RK2), (FP32, STEP_RK2), (FP64, STEP_AB2), (FP32, STEP_RK3)])
def test_checkpoint_restart_is_bit_exact(tmp_path, prec, stepop):
    """Save after 3 steps, continue 4 more; a run resumed from the file
    reproduces the continued run bit for bit (state, face B, AB history)."""
    s = ics.orszag_tang_3d(12, seed=2)
    prm = Params(12, 12, 12, precision=prec, stepop=stepop, tau=0.5 * ics.cfl_dt(s))
    path = tmp_path / "run.ckpt"
    with MHDSolver(prm, s) as a:
        a.step(3)
        a.save(path)
        ta, _ = a.step(4)
        fa = a.fetch()
    with MHDSolver.load(path, prm) as b:
        tb, _ = b.step(4)
        fb = b.fetch()
    assert ta == tb
    for k in FIELDS:
        assert np.array_equal(fa[k], fb[k]), k


@pytest.mark.parametrize("prec,stepop", [(FP32, STEP_RK2), (FP64, STEP_RK3)])
def test_batched_ensemble_equals_sequential(prec, stepop):
    """Uneven Cartesian PDM grids share one launch per kernel family; each
    grid's result is bit-identical to stepping it alone, over two calls (the
    second replays the cached graph) and with grids starting on different
    halves of their double-buffered state."""
    sizes = (16, 24, 8, 12, 32)
    states = [ics.orszag_tang_3d(n, seed=i, amp=0.5 + 0.3 * i, ny0=n + 2 * (i % 2)) for i, n in enumerate(sizes)]
    prms = [Params(n, n + 2 * (i % 2), n, precision=prec, stepop=stepop, tau=0.4 * ics.cfl_dt(st))
            for i, (n, st) in enumerate(zip(sizes, states))]
    seq = []
    for i, (prm, st) in enumerate(zip(prms, states)):
        with MHDSolver(prm, st) as g:
            g.step(1 + (i % 2) + 4)
            seq.append(g.fetch())
    ens = [MHDSolver(p, st) for p, st in zip(prms, states)]
    for i, e in enumerate(ens):  # odd grids one step ahead (the other buffer half for RK3)
        e.step(1 + (i % 2))
    ensemble_step(ens, 2)
    ensemble_step(ens, 2)
    for e, ref in zip(ens, seq):
        got = e.fetch()
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), k
        e.close()


def test_mixed_ensemble_uses_branches_and_matches():
    """A non-batchable ensemble (AB2 next to RK2) still equals sequential stepping."""
    s1, s2 = ics.orszag_tang_3d(12, seed=1), ics.orszag_tang_3d(10, seed=2)
    p1 = Params(12, 12, 12, stepop=STEP_AB2, tau=0.0)
    p2 = Params(10, 10, 10, stepop=STEP_RK2, tau=0.5 * ics.cfl_dt(s2))
    ref = []
    for p, s in ((p1, s1), (p2, s2)):
        with MHDSolver(p, s) as g:
            g.step(3)
            ref.append(g.fetch())
    ens = [MHDSolver(p1, s1), MHDSolver(p2, s2)]
    ensemble_step(ens, 3)
    for e, r in zip(ens, ref):
        got = e.fetch()
        for k in FIELDS:
            assert np.array_equal(got[k], r[k]), k
        e.close()


def test_autotuned_shapes_give_identical_steps():
    """Every launch shape the autotuner can pick computes the same bits."""
    s = ics.turbulence(32, seed=3)
    prm = Params(32, 32, 32, precision=FP32, tau=0.5 * ics.cfl_dt(s))
    with MHDSolver(prm, s) as a, MHDSolver(prm, s) as b:
        a.step(2)
        b.step(2)
        td, ey = b.autotune(reps=2)
        assert td in (4, 8, 16, 32) and ey in (1, 4, 8)
        a.step(3, graph=True)
        b.step(3, graph=True)
        fa, fb = a.fetch(), b.fetch()
    for k in FIELDS:
        assert np.array_equal(fa[k], fb[k]), k


def test_set_tiles_every_shape_gives_identical_steps():
    """mhd_set_tiles: all twelve FP32 PDM launch-shape pairs (face tiles 4,
    8, 16 and the 32-cell column sweeps; EMF as ei tiles 4x4, 8x8 or as slice
    streams) step to the same bits; fixed-shape handles refuse other shapes;
    mhd_device_info reports the device."""
    import ctypes as C
    from mhd3d_mpi_fortran_gb300 import abi
    from mhd3d_mpi_fortran_gb300.abi import MHDError
    s = ics.turbulence(40, seed=5)
    prm = Params(40, 40, 40, precision=FP32, tau=0.5 * ics.cfl_dt(s))
    ref = None
    for td in (4, 8, 16, 32):
        for ey in (4, 8, 1):
            with MHDSolver(prm, s) as g:
                g.set_tiles(td, ey)
                g.step(2)
                g.step(2, graph=True)
                f = g.fetch()
            if ref is None:
                ref = f
            for k in FIELDS:
                assert np.array_equal(f[k], ref[k]), (td, ey, k)
    with MHDSolver(Params(16, 16, 16, precision=FP64, tau=1e-3), ics.orszag_tang_3d(16)) as g:
        with pytest.raises(MHDError):
            g.set_tiles(16, 8)
    info = (C.c_int32 * 4)()
    assert abi.load().mhd_device_info(info) == 0
    assert info[0] > 0 and info[1] >= 10 and info[3] > 0


@pytest.mark.parametrize("shape,nord", [((33, 17, 9), 8), ((64, 40, 24), 8), ((16, 64, 33), 8), ((8, 8, 8), 8),
                                        ((40, 24, 20), 10)])
def test_streamed_emf_equals_tiles(shape, nord):
    """The slice-streamed EMF families (one edge column per thread along z for
    ei and ej, along y for ek; the last edge row of the in-slice transverse
    axis in a separate launch) against the shared-memory tiles: every EMF,
    and the state after RK2 steps, bit-identical on ragged grids whose x
    extent is not a multiple of the 32-lane tile, whose stream axis spans one
    or several segments, a grid smaller than one tile, and 5 ghost layers
    (the slices keep the 4-cell stencil halo whatever the ghost depth)."""
    s = rand_state(*shape, seed=sum(shape) + 1, nord=nord)
    prm = Params(*shape, precision=FP32, tau=2e-4, nord=nord)
    out = {}
    for ey in (8, 1):
        with MHDSolver(prm, s) as g:
            g.set_tiles(8, ey)
            e = g.debug_emf()
            g.step(3)
            out[ey] = (e, g.fetch())
    for k in range(3):
        assert np.array_equal(out[8][0][k], out[1][0][k]), k
    for k in FIELDS:
        assert np.array_equal(out[8][1][k], out[1][1][k]), k


@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK3])
def test_column_sweeps_equal_face_tiles_for_ab2_and_rk3(stepop):
    """The z-sweep epilogue applies every stepper's stage combine exactly as
    the z-face tiles do: FP32 PDM AB2 and RK3 steps are bit-identical."""
    s = ics.turbulence(40, seed=8)
    prm = Params(40, 40, 40, stepop=stepop, precision=FP32, tau=0.4 * ics.cfl_dt(s))
    out = {}
    for td in (8, 32):
        with MHDSolver(prm, s) as g:
            g.set_tiles(td, 8)
            g.step(3)
            out[td] = g.fetch()
    for k in FIELDS:
        assert np.array_equal(out[8][k], out[32][k]), k


@pytest.mark.parametrize("recon", [2, 3, 4, 5])
def test_weno_column_sweeps_equal_face_tiles(recon):
    """FP32 TVD, WENO5, MP-WENO5, TVD-MC: the column-sweep face kernels (shape
    32, the default) and the 8-cell face tiles step to the same bits."""
    s = ics.turbulence(40, seed=6)
    prm = Params(40, 40, 40, reconop=recon, precision=FP32, tau=0.4 * ics.cfl_dt(s))
    out = {}
    for td in (8, 32):
        with MHDSolver(prm, s) as g:
            g.set_tiles(td, 8)
            g.step(3)
            out[td] = g.fetch()
    for k in FIELDS:
        assert np.array_equal(out[8][k], out[32][k]), k


@pytest.mark.parametrize("ey", [8, 1])
def test_batched_column_sweeps_equal_sequential_tiles(ey):
    """Batched ensemble on the column-sweep face kernels (tile 32) and the
    8x8 ei EMF tiles or the slice-streamed EMF against each grid stepped
    alone on its default shapes: bit-identical."""
    sizes = (16, 40, 24)
    states = [ics.turbulence(n, seed=10 + i) for i, n in enumerate(sizes)]
    prms = [Params(n, n, n, precision=FP32, tau=0.4 * ics.cfl_dt(st)) for n, st in zip(sizes, states)]
    seq = []
    for prm, st in zip(prms, states):
        with MHDSolver(prm, st) as g:
            g.step(4)
            seq.append(g.fetch())
    ens = [MHDSolver(p, st) for p, st in zip(prms, states)]
    for e in ens:
        e.set_tiles(32, ey)
    ensemble_step(ens, 4)
    for e, ref in zip(ens, seq):
        got = e.fetch()
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), k
        e.close()


def test_ensemble_autotune_then_step_equals_sequential():
    from mhd3d_mpi_fortran_gb300 import ensemble_autotune
    sizes = (16, 20, 12)
    states = [ics.orszag_tang_3d(n, seed=i) for i, n in enumerate(sizes)]
    prms = [Params(n, n, n, precision=FP32, tau=0.5 * ics.cfl_dt(st)) for n, st in zip(sizes, states)]
    seq = []
    for prm, st in zip(prms, states):
        with MHDSolver(prm, st) as g:
            g.step(3)
            seq.append(g.fetch())
    ens = [MHDSolver(p, st) for p, st in zip(prms, states)]
    td, ey = ensemble_autotune(ens, reps=2)
    assert td in (4, 8, 16) and ey in (1, 4, 8)
    ensemble_step(ens, 3)
    for e, ref in zip(ens, seq):
        got = e.fetch()
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), k
        e.close()


# ---- Yee edge EMF (get_eijk_Yee; commented out in the reference) ----------
@pytest.mark.parametrize("recon", RECONS)
@pytest.mark.parametrize("shape", [(11, 12, 10), (33, 16, 8)])
def test_yee_emf_fp64_match_oracle(recon, shape):
    from mhd3d_mpi_fortran_gb300.abi import EMF_YEE
    s = rand_state(*shape, seed=20 + recon)
    prm = Params(*shape, reconop=recon, emf=EMF_YEE, tau=1e-3)
    with MHDSolver(prm, s) as gpu:
        eg = gpu.debug_emf()
    eo = OracleSolver(prm, s).emf()
    for e in range(3):
        assert relmax(eg[e], eo[e]) <= 1e-13, e


@pytest.mark.parametrize("stepop", [STEP_AB2, STEP_RK2, STEP_RK3])
@pytest.mark.parametrize("recon", [1, 4])
def test_yee_steps_fp64_match_oracle(stepop, recon):
    from mhd3d_mpi_fortran_gb300.abi import EMF_YEE
    s = ics.orszag_tang_3d(12, seed=7, ny0=10, nz0=9)
    prm = Params(12, 10, 9, reconop=recon, stepop=stepop, emf=EMF_YEE, tau=0.4 * ics.cfl_dt(s))
    with MHDSolver(prm, s) as gpu:
        tg, sg = gpu.step(4)
        fg = gpu.fetch()
        dg = gpu.diagnostics()
    o = OracleSolver(prm, s)
    to, so = o.step(4)
    fo = o.fetch()
    assert tg == pytest.approx(to, rel=1e-13) and sg == so
    for k in FIELDS:
        assert relmax(fg[k], fo[k]) <= 1e-11, k
    assert dg["divb_max"] <= 1e-12


def test_yee_fp32_budget_and_cartesian_only():
    from mhd3d_mpi_fortran_gb300.abi import EMF_YEE, MHDError
    s = ics.orszag_tang_3d(32, seed=0)
    tau = ics.cfl_dt(s)
    res = {}
    for prec in (FP64, FP32):
        with MHDSolver(Params(32, 32, 32, precision=prec, emf=EMF_YEE, tau=tau), s) as gpu:
            gpu.step(20)
            res[prec] = gpu.fetch()
    for k in ("rho", "p", "vx", "bi"):
        a, b = res[FP32][k], res[FP64][k]
        assert np.abs(a - b).sum() / np.abs(b).sum() <= 1e-5, k
    m = ics.mapped_blast(8)
    with pytest.raises(MHDError):
        MHDSolver(Params(8, 8, 8, emf=EMF_YEE, tau=0.0, stepop=STEP_AB2), m)


def test_fetch_fills_caller_arrays_in_place():
    s = ics.orszag_tang_3d(12, seed=1)
    with MHDSolver(Params(12, 12, 12, tau=0.4 * ics.cfl_dt(s)), s) as g:
        g.step(2)
        a = g.fetch()
        dst = g.output_arrays()
        for v in dst.values():
            v.fill(7.0)
        b = g.fetch(out=dst)
    assert b is dst
    for k in FIELDS:
        assert np.array_equal(a[k], dst[k]), k


def test_step_tau_inout_sets_the_fixed_rk_dt():
    """mhd_step reads the driver's tau: for RK with the deck dt a changed
    positive tau becomes the fixed dt before the step (bit-identical to
    mhd_set_tau then mhd_step), an unchanged one is a no-op; AB2 takes its CFL
    dt and ignores the input, as step_ab overwrites tau (mhd3d3.f90:3609)."""
    s = ics.orszag_tang_3d(12, seed=3)
    t0 = 0.4 * ics.cfl_dt(s)
    t1 = 0.7 * t0
    prm = Params(12, 12, 12, tau=t0)
    with MHDSolver(prm, s) as a, MHDSolver(prm, s) as b:
        lib = a.lib
        tau, st = C.c_double(t0), C.c_uint32()
        for _ in range(2):
            assert lib.mhd_step(a.h, C.byref(tau), C.byref(st)) == E_OK
            assert tau.value == t0
        tau.value = t1
        assert lib.mhd_step(a.h, C.byref(tau), C.byref(st)) == E_OK
        assert tau.value == t1
        assert lib.mhd_step(a.h, C.byref(tau), C.byref(st)) == E_OK
        assert tau.value == t1
        b.step(2)
        b.set_tau(t1)
        b.step(2)
        fa, fb = a.fetch(), b.fetch()
    for k in FIELDS:
        assert np.array_equal(fa[k], fb[k]), k
    pab = Params(12, 12, 12, stepop=STEP_AB2, tau=3e-4)
    with MHDSolver(pab, s) as a, MHDSolver(pab, s) as b:
        tau = C.c_double(123.0)
        assert a.lib.mhd_step(a.h, C.byref(tau), None) == E_OK
        tb, _ = b.step(1)
        assert tau.value == tb and tau.value < 1.0
