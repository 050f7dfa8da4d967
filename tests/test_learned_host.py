"""Host side of the learned correction: restriction, magnetic targets and
feature layout (no GPU)."""
import numpy as np

from mhd3d_mpi_fortran_gb300 import ics, learned


def _fine_dict(n=16, seed=1):
    s = ics.orszag_tang_3d(n, seed=seed)
    d = learned.state_dict(s)
    # fill periodic ghosts so every interior cell is defined
    return d, s


def test_restriction_conserves_and_keeps_div_b_zero():
    d, s = _fine_dict(16)
    c = learned.restrict(d, 16)
    ng = 4
    Uf = learned.conserved(d, ng)
    Uc = learned.conserved(learned.state_dict(c), ng)
    assert np.allclose(Uf[:5].sum(axis=(1, 2, 3)) / 8.0, Uc[:5].sum(axis=(1, 2, 3)), rtol=1e-12, atol=1e-12)
    n, dx = 8, 1.0 / 8
    sl = (slice(ng, ng + n),) * 3
    bi, bj, bk = c.bi, c.bj, c.bk
    div = ((bi[ng + 1:ng + n + 1, ng:ng + n, ng:ng + n] - bi[sl]) + (bj[ng:ng + n, ng + 1:ng + n + 1, ng:ng + n] - bj[sl])
           + (bk[ng:ng + n, ng:ng + n, ng + 1:ng + n + 1] - bk[sl])) / dx
    assert np.abs(div).max() <= 1e-12


def test_potential_fit_reproduces_face_increments_made_by_the_apply_operator():
    rng = np.random.default_rng(0)
    n, dx = 8, 0.125
    A = rng.standard_normal((3, n, n, n))
    faces = learned.curl_faces(A, dx)
    A2 = learned.potential_from_faces(*faces, dx=dx)
    again = learned.curl_faces(A2, dx)
    for a, b in zip(faces, again):
        assert np.abs(a - b).max() <= 1e-10 * np.abs(a).max()


def test_feature_rows_are_the_normalised_3x3x3_stencil():
    rng = np.random.default_rng(2)
    n = 5
    U = rng.standard_normal((8, n, n, n))
    mean, std = rng.standard_normal(8), 1.0 + rng.random(8)
    x = learned.bf16_bits(np.zeros(1))  # dtype check
    bits = learned.features(U, mean, std)
    vals = (bits.astype(np.uint32) << 16).view(np.float32)
    i, j, k = 4, 0, 2
    row = vals[i + n * (j + n * k)]
    f = 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                ref = (U[:, (i + dx) % n, (j + dy) % n, (k + dz) % n] - mean) / std
                assert np.allclose(row[f:f + 8], ref, rtol=2 ** -8, atol=1e-6)
                f += 8
    assert np.all(row[216:] == 0) and x.dtype == np.uint16


def test_choose_damping_picks_the_smallest_rollout_error():
    errs = {1.0: 1.03, 0.75: 0.88, 0.5: 0.86, 0.25: 0.91}
    g, got = learned.choose_damping(lambda g: errs[g])
    assert g == 0.5 and got == errs


class _FakeMLP:
    """Stands in for the GPU network: records the output scales it is given."""

    def __init__(self):
        self.norm = None
        self.calls = []

    def set_norm(self, mean, std, scale):
        self.norm = [np.asarray(mean, np.float32), np.asarray(std, np.float32), np.asarray(scale, np.float32)]
        self.calls.append(float(self.norm[2][0]))


def test_damp_scales_the_outputs_and_keeps_the_best(monkeypatch):
    mlp = _FakeMLP()
    mlp.set_norm(np.zeros(8), np.ones(8), np.full(8, 2.0))
    mlp.calls.clear()
    # a rollout error that is smallest when the output scale is 1.5 (gamma 0.75)
    monkeypatch.setattr(learned, "evaluate",
                        lambda m, seed, n, steps, nord=8: {"corrected_l1": abs(float(m.norm[2][0]) - 1.5)})
    g, errs = learned.damp(mlp, seed=3, n_coarse=16, steps=10)
    assert g == 0.75
    assert mlp.calls[:4] == [2.0, 1.5, 1.0, 0.5]          # each damping tried on the undamped scales
    assert np.allclose(mlp.norm[2], 1.5)                  # the chosen one is left in place
    assert set(errs) == set(learned.DAMPINGS)
