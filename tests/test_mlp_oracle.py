"""The MLP oracle's backward pass against finite differences (CPU, FP64)."""
import numpy as np

from oracle import mlp_oracle as mo


def _data(n=40, seed=0):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, mo.FIN))
    x[:, :216] = rng.standard_normal((n, 216))
    t = rng.standard_normal((n, mo.NOUT)) * 0.3
    return x, t


def test_gradient_matches_central_differences():
    x, t = _data()
    p = mo.init_params(3).astype(np.float64)
    _, g = mo.loss_and_grad(p, x, t, bf16=False)
    rng = np.random.default_rng(1)
    w = mo.unpack(np.arange(mo.NPARAM))
    # coordinates in every block (W1 used columns, biases, W3 used rows)
    picks = [int(w["W1"][5, 17]), int(w["W1"][63, 215]), int(w["b1"][9]), int(w["W2"][3, 40]), int(w["b2"][60]),
             int(w["W3"][7, 2]), int(w["b3"][4])] + list(rng.integers(0, int(w["W1"][0, 200]), 5))
    for i in picks:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_and_grad(pp, x, t, bf16=False)[0] - mo.loss_and_grad(pm, x, t, bf16=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])


def test_padding_gets_no_gradient():
    x, t = _data()
    _, g = mo.loss_and_grad(mo.init_params(2), x, t)
    w = mo.unpack(g)
    assert np.all(w["W1"][:, 216:] == 0) and np.all(w["W3"][8:] == 0) and np.all(w["b3"][8:] == 0)


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], dtype=np.float32)
    got = mo.bf16_val(mo.bf16_bits(v))
    assert got[0] == 1.0 and got[1] == 1.0  # tie to even
    assert got[2] == 1.0078125 and got[3] == -2.5
    assert abs(got[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8
