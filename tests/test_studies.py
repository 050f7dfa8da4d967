"""Host-side helpers of the accuracy studies (no GPU)."""
import numpy as np

from mhd3d_mpi_fortran_gb300 import ics, studies


def _state_dict(n, ng=4):
    sh = (n + 2 * ng,) * 3
    return {k: np.zeros(sh, order="F") for k in studies.FIELDS}


def test_spectrum_puts_a_single_mode_in_its_shell():
    n, ng = 16, 4
    f = _state_dict(n, ng)
    f["rho"][...] = 1.0
    x = (np.arange(n) + 0.5) / n
    f["vx"][ng:-ng, ng:-ng, ng:-ng] = np.sin(2 * np.pi * 3 * x)[None, :, None]
    e = studies.spectrum(f, ng)
    assert np.argmax(e) == 2  # shell k = 3 (index k-1)
    assert abs(e.sum() - 0.25) < 1e-12  # Parseval: mean of rho v^2 / 2


def test_errors_are_zero_for_identical_states_and_grouped():
    s = ics.orszag_tang_3d(8)
    f = {k: getattr(s, k) for k in ("rho", "vx", "vy", "vz", "p")}
    for k in ("bx", "by", "bz"):
        f[k] = np.ones_like(s.rho)
    g = {k: v.copy() for k, v in f.items()}
    e = studies.errors(g, f, 4)
    assert all(v["l1"] == 0.0 and v["l2"] == 0.0 for v in e.values())
    g["vz"] = g["vz"] + 1e-3
    e = studies.errors(g, f, 4)
    assert 0 < e["v"]["l1"] < 1e-2 and e["rho"]["l1"] == 0.0


def test_coarsen_keeps_mass_and_div_free_faces():
    from mhd3d_mpi_fortran_gb300.learned import state_dict
    n, ng = 16, 4
    s = ics.turbulence(n, seed=3)
    f = state_dict(s)
    c = studies.coarsen(f, n, 2)
    m = n // 4
    inner = (slice(ng, ng + m),) * 3
    assert c["rho"].shape == (m + 2 * ng,) * 3
    assert np.isclose(c["rho"][inner].mean(), s.rho[ng:-ng, ng:-ng, ng:-ng].mean(), rtol=1e-13)
    bi, bj, bk = c["bi"], c["bj"], c["bk"]
    div = (bi[ng + 1:ng + m + 1, ng:ng + m, ng:ng + m] - bi[ng:ng + m, ng:ng + m, ng:ng + m]
           + bj[ng:ng + m, ng + 1:ng + m + 1, ng:ng + m] - bj[ng:ng + m, ng:ng + m, ng:ng + m]
           + bk[ng:ng + m, ng:ng + m, ng + 1:ng + m + 1] - bk[ng:ng + m, ng:ng + m, ng:ng + m])
    assert np.abs(div).max() <= 1e-12 * np.abs(bi).max()
