"""GPU parity of the curvilinear metric mode (mhd_init_mapped) against the
oracle's metric mode, through the C ABI.

FP64 metric mode follows the oracle's expression order with no FMA (the
metric terms are computed on the device by the same formulas), so results
agree to a few ulps apart from exp/erfc.  Errors of the vector fields are
normalised by the largest component of their group (v, cell B, face flux).
"""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import ics, MHDSolver
from mhd3d_mpi_fortran_gb300.abi import (Params, BC_OUTFLOW, BC_PERIODIC, STEP_AB2, STEP_RK2, STEP_RK3, FP32,
                                         FP64, DT_CFL, E_ARG, MHDError)
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

GROUPS = (("rho",), ("p",), ("vx", "vy", "vz"), ("bx", "by", "bz"), ("bi", "bj", "bk"))


def group_err(a: dict, b: dict) -> dict:
    out = {}
    for grp in GROUPS:
        scale = max(np.abs(b[k]).max() for k in grp)
        for k in grp:
            out[k] = np.abs(a[k] - b[k]).max() / max(scale, 1e-300)
    return out


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def ot(seed=0):
    return ics.mapped_orszag_tang(12, seed=seed, ny0=10, nz0=9)


@pytest.mark.parametrize("recon", [1, 2, 3, 4, 5])
def test_metric_fluxes_fp64_match_oracle(recon):
    s = ot(recon)
    prm = Params(12, 10, 9, reconop=recon, tau=1e-3)
    with MHDSolver(prm, s) as gpu:
        fg = gpu.debug_fluxes()
    fo = OracleSolver(prm, s).fluxes()
    for d in range(3):
        for q in range(8):
            assert relmax(fg[d][q], fo[d][q]) <= 1e-13, (d, q)


@pytest.mark.parametrize("recon", [1, 2, 3, 4, 5])
def test_metric_emf_fp64_match_oracle(recon):
    s = ot(10 + recon)
    prm = Params(12, 10, 9, reconop=recon, tau=1e-3)
    with MHDSolver(prm, s) as gpu:
        eg = gpu.debug_emf()
    eo = OracleSolver(prm, s).emf()
    for e in range(3):
        assert relmax(eg[e], eo[e]) <= 1e-13, e


@pytest.mark.parametrize("recon,stepop", [(1, STEP_RK2), (1, STEP_AB2), (1, STEP_RK3), (2, STEP_RK2),
                                          (3, STEP_AB2), (4, STEP_RK2), (5, STEP_RK3)])
def test_metric_steps_fp64_match_oracle(recon, stepop):
    s = ot(recon)
    prm = Params(12, 10, 9, reconop=recon, stepop=stepop, tau=0.5 * ics.cfl_dt_mapped(s))
    with MHDSolver(prm, s) as gpu:
        tg, sg = gpu.step(4)
        fg = gpu.fetch()
    o = OracleSolver(prm, s)
    to, so = o.step(4)
    fo = o.fetch()
    assert tg == pytest.approx(to, rel=1e-13)
    assert sg == so
    for k, e in group_err(fg, fo).items():
        assert e <= 1e-11, (k, e)


def test_metric_blast_outflow_ab2_fp64():
    """The curvilinear blast (sine mapping, outflow walls, PDM, AB2) at 16^3."""
    s = ics.mapped_blast(16)
    prm = Params(16, 16, 16, stepop=STEP_AB2, bc=(BC_OUTFLOW,) * 3, tau=0.0)
    with MHDSolver(prm, s) as gpu:
        tg, _ = gpu.step(6)
        fg = gpu.fetch()
        dg = gpu.diagnostics()
    o = OracleSolver(prm, s)
    to, _ = o.step(6)
    fo = o.fetch()
    do = o.diagnostics()
    assert tg == pytest.approx(to, rel=1e-12)
    for k, e in group_err(fg, fo).items():
        assert e <= 1e-11, (k, e)
    assert dg["mass"] == pytest.approx(do["mass"], rel=1e-13)
    assert dg["energy"] == pytest.approx(do["energy"], rel=1e-12)
    assert dg["divb_max"] <= 1e-12


def test_metric_cfl_mode_and_diagnostics():
    s = ics.mapped_orszag_tang(14, seed=3)
    prm = Params(14, 14, 14, dt_mode=DT_CFL, tau=1.0)
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
    assert dg["mass"] == pytest.approx(dg0["mass"], rel=1e-13)  # periodic: conserved
    assert dg["energy"] == pytest.approx(do["energy"], rel=1e-12)
    assert dg["divb_max"] <= 1e-12 and do["divb_max"] <= 1e-12


def test_metric_fp32_error_budget_and_div_b():
    """FP32 state and fluxes with the FP64 metric against the FP64 solution on
    the curvilinear blast (outflow, PDM, AB2)."""
    s = ics.mapped_blast(24)
    prm = dict(stepop=STEP_AB2, bc=(BC_OUTFLOW,) * 3, tau=0.0)
    res, diag = {}, {}
    for prec in (FP64, FP32):
        with MHDSolver(Params(24, 24, 24, precision=prec, **prm), s) as gpu:
            gpu.step(20)
            res[prec] = gpu.fetch()
            diag[prec] = gpu.diagnostics()
    for k in ("rho", "p", "bx"):
        a, b = res[FP32][k], res[FP64][k]
        l1 = np.abs(a - b).sum() / np.abs(b).sum()
        assert l1 <= 1e-5, (k, l1)
    assert diag[FP32]["divb_max"] <= 1e-4
    assert diag[FP64]["divb_max"] <= 1e-12


def test_metric_graph_equals_stream_fp64():
    s = ot(2)
    prm = Params(12, 10, 9, tau=0.5 * ics.cfl_dt_mapped(s))
    with MHDSolver(prm, s) as a, MHDSolver(prm, s) as b:
        a.step(4)
        b.step(2, graph=True)
        b.step(2, graph=True)
        fa, fb = a.fetch(), b.fetch()
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k


@pytest.mark.parametrize("prec,stepop", [(FP64, STEP_RK2), (FP32, STEP_AB2)])
def test_metric_checkpoint_restart_is_bit_exact(tmp_path, prec, stepop):
    s = ot(4)
    prm = Params(12, 10, 9, precision=prec, stepop=stepop, tau=0.5 * ics.cfl_dt_mapped(s))
    path = tmp_path / "mapped.ckpt"
    with MHDSolver(prm, s) as a:
        a.step(3)
        a.save(path)
        ta, _ = a.step(3)
        fa = a.fetch()
    with MHDSolver.load(path, prm) as b:
        tb, _ = b.step(3)
        fb = b.fetch()
    assert ta == tb
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k


def test_mapped_grid_with_inverted_cells_is_rejected():
    s = ics.mapped_blast(8)
    X, Y, Z = s.nodes
    s.nodes = (np.asfortranarray(X[::-1, :, :]), Y, Z)  # mirrored x: negative volumes
    with pytest.raises(MHDError) as e:
        MHDSolver(Params(8, 8, 8, tau=1e-3), s)
    assert e.value.code == E_ARG
