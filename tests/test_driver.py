"""Driver loop output formats (CPU) and a short deck run on the GPU."""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import driver, ics

DECK = """
 &dom
 xmin=-1., xmax=1., ymin=-1., ymax=1., zmin=-1., zmax=1.
/
 &grid
 nx0G=8, ny0G=8, nz0G=16, xprocs=1, yprocs=1, zprocs=1
/
 &comset
 nord=8, reconop=4, stepop=3, outop=2
/
 &list
 nts=3, tau=0.002, nframes=2, nrst=0, nfdump=10
/
 &free
 cfl=.3, pdmb=4., eps=1.e-8, alpha=2., beta=4.
/
"""


def test_stime_records_are_fortran_unformatted(tmp_path):
    path = tmp_path / "stime.out"
    path.write_bytes(b"".join(driver.fortran_record(np.float64(t).tobytes()) for t in (0.0, 0.25, 0.5)))
    raw = path.read_bytes()
    assert len(raw) == 3 * 16 and raw[:4] == (8).to_bytes(4, "little") and raw[12:16] == (8).to_bytes(4, "little")
    assert np.array_equal(driver.read_stime(path), [0.0, 0.25, 0.5])


def test_frames_use_the_hdf5_dataset_layout(tmp_path):
    s = ics.shock_tube(16, axis=2, ntrans=8)
    f = {k: getattr(s, k) for k in ("rho", "vx", "vy", "vz", "p")}
    f.update(bx=s.rho * 2, by=s.rho * 3, bz=s.p * 5)
    w = driver.FrameWriter(tmp_path, (8, 8, 16), 1, 4)
    w.write(f, 0.0)
    w.write(f, 0.1)
    w.close(2)
    fr = driver.read_frames(tmp_path)
    assert fr["rho"].shape == (2, 16, 8, 8)
    x, y, z = 3, 5, 11
    assert fr["p"][1, z, y, x] == s.p[4 + x, 4 + y, 4 + z]
    assert np.array_equal(fr["time"], [0.0, 0.1])
    assert np.array_equal(driver.read_stime(tmp_path / "stime.out"), [0.0, 0.1])


def test_initial_state_is_the_reference_tube():
    deck = driver.read_deck(DECK)
    s = driver.initial_state(deck, 8)
    assert s.rho.shape == (16, 16, 24)
    assert s.rho[8, 8, 5] == 1.0 and s.rho[8, 8, 20] == 0.125


# mhd3d2.in's scheme and grid (one rank, a smaller x-y grid): 2-D, nz0 = 1
DECK2 = """
 &dom
 xmin=0., xmax=1., ymin=0., ymax=1., zmin=0., zmax=1.
/
 &grid
 nx0G=16, ny0G=16, nz0=1, xprocs=1, yprocs=1
/
 &comset
 nord=6, reconop=4, stepop=3, outop=2
/
 &list
 nts=100, tau=1.e-4, nframes=2000, nrst=0, nfdump=10
/
 &free
 cfl=.3, pdmb=4., eps=1.e-8, alpha=2., beta=4.
/
"""


def test_mhd3d2_ics_lift_z_to_eight_planes_with_the_z_constant_fill():
    from mhd3d_mpi_fortran_gb300.abi import BC_OUTFLOW, BC_PERIODIC
    deck = driver.read_deck(DECK2)
    assert driver.ic_grid(deck, 6, "otv") == (16, 16, 8, (BC_PERIODIC, BC_PERIODIC, BC_OUTFLOW))
    s = driver.initial_state(deck, 6, "otv")
    ref = ics.orszag_tang_2d(16, nz0=8, nord=6)
    for a, b in zip(s.arrays(), ref.arrays()):
        assert np.array_equal(a, b)
    assert driver.initial_state(deck, 6, "imp").rho.shape == (22, 22, 14)
    assert driver.initial_state(deck, 6, "bws").bi[0, 0, 0] == 0.5
    with pytest.raises(ValueError):
        driver.ic_grid(deck, 6, "nope")


def test_mhd3d2_deck_stays_two_dimensional():
    """init_ic_otv with mhd3d2.in's scheme (MP-WENO5, RK3, nord 6) on the lifted
    grid: every z plane evolves identically, as in the reference's 2-D run."""
    from mhd3d_mpi_fortran_gb300.deck import params_from_deck
    from oracle.oracle import OracleSolver
    deck = driver.read_deck(DECK2)
    prm = params_from_deck(deck)
    _, _, prm.nz0, prm.bc = driver.ic_grid(deck, prm.nord, "otv")
    o = OracleSolver(prm, driver.initial_state(deck, prm.nord, "otv"))
    _, st = o.step(5)
    assert st == 0
    out = o.fetch()
    for k in ("rho", "p", "vx", "vy", "bi", "bj"):
        a = out[k]
        for z in range(1, a.shape[2]):
            assert np.array_equal(a[:, :, z], a[:, :, 0]), (k, z)
    assert np.abs(out["vz"]).max() == 0.0 and np.abs(out["bk"]).max() == 0.0


@pytest.mark.gpu
def test_deck_run_writes_every_frame(tmp_path):
    out = driver.run(DECK, tmp_path)
    assert out["frames"] == 3 and out["stopped"] is None
    fr = driver.read_frames(tmp_path)
    assert fr["rho"].shape == (3, 16, 8, 8)
    assert np.allclose(fr["time"], [0.0, 3 * 0.002, 6 * 0.002])
    assert np.array_equal(driver.read_stime(tmp_path / "stime.out"), fr["time"])
    s0 = driver.initial_state(driver.read_deck(DECK), 8)
    assert np.array_equal(fr["rho"][0], s0.rho[4:-4, 4:-4, 4:-4].transpose(2, 1, 0))
    assert not np.array_equal(fr["rho"][2], fr["rho"][0])


@pytest.mark.parametrize("recon,stepop,bc", [(4, 3, "2d"), (3, 1, "walls"), (5, 2, "2d")])
def test_nord6_and_nord8_give_the_same_interior(recon, stepop, bc):
    """Oracle property: WENO / TVD stencils reach 3 cells, so a 4th ghost layer
    (an exact copy: periodic, outflow, mirror) changes neither the interior
    nor the time steps, bit for bit."""
    from mhd3d_mpi_fortran_gb300.abi import BC_EVEN, BC_OUTFLOW, BC_PERIODIC, Params
    from oracle.oracle import OracleSolver
    bcs = (BC_PERIODIC, BC_PERIODIC, BC_OUTFLOW) if bc == "2d" else (BC_EVEN,) * 3
    res = {}
    for nord in (6, 8):
        ng = nord // 2
        prm = Params(16, 16, 8, nord=nord, reconop=recon, stepop=stepop, bc=bcs, tau=1e-3 if stepop == 1 else 2e-3)
        o = OracleSolver(prm, ics.orszag_tang_2d(16, nz0=8, nord=nord))
        taus = [o.step(1)[0] for _ in range(3)]
        out = o.fetch()
        res[nord] = (taus, {k: a[ng:a.shape[0] - ng, ng:a.shape[1] - ng, ng:a.shape[2] - ng] for k, a in out.items()})
    assert res[6][0] == res[8][0]
    for k in res[6][1]:
        assert np.array_equal(res[6][1][k], res[8][1][k]), k


@pytest.mark.gpu
def test_mhd3d2_otv_deck_runs_on_the_gpu(tmp_path):
    """mhd3d2.in's scheme (MP-WENO5, RK3) at its own ghost depth (nord 6) from
    init_ic_otv on the lifted 2-D grid, through the driver loop: the last frame
    matches the oracle's FP64 run, and every z plane of it is the same."""
    from mhd3d_mpi_fortran_gb300.deck import params_from_deck
    from oracle.oracle import OracleSolver
    deck = driver.read_deck(DECK2)
    out = driver.run(deck, tmp_path, nframes=2, nts=3, ic="otv")
    assert out["frames"] == 3 and out["stopped"] is None
    fr = driver.read_frames(tmp_path)
    assert fr["rho"].shape == (3, 8, 16, 16)
    prm = params_from_deck(deck)
    assert prm.nord == 6
    _, _, prm.nz0, prm.bc = driver.ic_grid(deck, prm.nord, "otv")
    o = OracleSolver(prm, driver.initial_state(deck, prm.nord, "otv"))
    o.step(6)
    ref = o.fetch()
    for v in ("rho", "vx", "vy", "p", "bx", "by"):
        want = ref[v][3:-3, 3:-3, 3:-3].transpose(2, 1, 0)
        got = fr[v][2]
        assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max(), v
        for z in range(1, got.shape[0]):
            assert np.array_equal(got[z], got[0]), (v, z)
