"""Tensor-core (tcgen05) kernels of the learned coarse-grid correction,
checked through the C ABI against the numpy oracle (oracle/mlp_oracle.py),
and the correction coupled to the solver."""
import numpy as np
import pytest

from mhd3d_mpi_fortran_gb300 import abi, ics, learned, MHDSolver
from mhd3d_mpi_fortran_gb300.abi import Params, FP32
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 64, 256), (300, 16, 64), (256, 64, 128), (128, 256, 16)])
def test_tc_gemm_matches_fp32_product_of_bf16_operands(M, N, K):
    lib = abi.load()
    rng = np.random.default_rng(M + N + K)
    a = mo.bf16_bits(rng.standard_normal((M, K)))
    b = mo.bf16_bits(rng.standard_normal((N, K)))
    c = np.zeros((M, N), dtype=np.float32)
    rc = lib.mhd_tc_gemm_test(a.ctypes.data, b.ctypes.data, c.ctypes.data, M, N, K)
    assert rc == 0, lib.mhd_last_error()
    ref = mo.bf16_val(a) @ mo.bf16_val(b).T
    # exact BF16 products, FP32 accumulation
    assert np.abs(c - ref).max() <= 1e-5 * np.abs(ref).max() + 1e-5


def _features(n, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, mo.FIN), dtype=np.float32)
    x[:, :216] = rng.standard_normal((n, 216))
    return mo.bf16_bits(x)


def test_forward_matches_oracle():
    p = mo.init_params(1)
    xb = _features(300, 2)
    mlp = learned.MLP(p)
    y = mlp.forward(xb)
    ref = mo.forward(p, mo.bf16_val(xb), bf16=True)
    # only FP32 accumulation order (and the BF16 roundings it can flip) differ
    assert np.abs(y - ref).max() <= 1e-2 * np.abs(ref).max()
    assert np.sqrt(np.mean((y - ref) ** 2)) <= 2e-3 * np.sqrt(np.mean(ref ** 2))
    mlp.close()


def test_gradient_matches_oracle():
    """Gradients of the tensor-core backward pass (all weight gradients are
    tcgen05 GEMMs) against the oracle with the same BF16 rounding points."""
    p = mo.init_params(4)
    n = 384
    xb = _features(n, 5)
    t = (np.random.default_rng(6).standard_normal((n, mo.NOUT)) * 0.5).astype(np.float32)
    mlp = learned.MLP(p)
    mlp.set_data(xb, t)
    loss, g = mlp.grad(0, n)
    lref, gref = mo.loss_and_grad(p, mo.bf16_val(xb), t, bf16=True)
    assert loss == pytest.approx(lref, rel=1e-3)
    gw, gr = mo.unpack(g), mo.unpack(gref)
    for name, _ in mo.SHAPES:
        a, b = gw[name], gr[name]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel <= 2e-2, (name, rel)
    mlp.close()


def test_training_reduces_the_loss():
    rng = np.random.default_rng(7)
    n = 8192
    x = np.zeros((n, mo.FIN), dtype=np.float32)
    x[:, :216] = rng.standard_normal((n, 216))
    wt = rng.standard_normal((216, mo.NOUT)) / np.sqrt(216)
    t = np.tanh(x[:, :216] @ wt).astype(np.float32)
    mlp = learned.MLP(mo.init_params(8))
    xb = mo.bf16_bits(x)
    mlp.set_data(xb, t)
    l0, _ = mlp.grad(0, 1024)
    loss = mlp.train(300, batch=1024, lr=2e-3, seed=1)
    l1, _ = mlp.grad(0, 1024)
    assert l1 < 0.25 * l0, (l0, l1, loss)
    mlp.close()


def test_correction_keeps_div_b_and_a_zero_network_is_the_identity():
    s = ics.turbulence(16, seed=2)
    prm = Params(16, 16, 16, precision=FP32, tau=0.5 * ics.cfl_dt(s))
    zero = learned.MLP(np.zeros(learned.NPARAM, dtype=np.float32))
    small = learned.MLP(learned.init_params(3) * 0.1)
    small.set_norm(np.zeros(8), np.ones(8), np.full(8, 1e-2))
    with MHDSolver(prm, s) as a, MHDSolver(prm, s) as b, MHDSolver(prm, s) as c:
        d0 = c.diagnostics()
        a.step(4)
        zero.step_corrected(b, 4)
        _, st = small.step_corrected(c, 4)
        fa, fb = a.fetch(), b.fetch()
        dc = c.diagnostics()
    for k in ("rho", "vx", "p", "bi"):
        assert np.abs(fa[k] - fb[k]).max() <= 1e-5 * np.abs(fa[k]).max(), k
    assert st == 0
    # the magnetic correction is a curl (div-free), the hydro one has zero mean
    assert dc["divb_max"] <= 1e-4
    assert dc["mass"] == pytest.approx(d0["mass"], rel=1e-6)
    zero.close()
    small.close()


def test_trained_correction_reduces_coarse_error():
    """Small version of the learned-correction study: pairs from four fine
    32^3 runs, outputs calibrated on a fifth, evaluated on a held-out sixth
    seed over 8 coarse 16^3 steps.  The corrected coarse run is closer to the
    restricted fine run than the plain coarse run."""
    mlp, loss, npairs, alpha = learned.train_correction([11, 12, 13, 14], 16, steps=40, every=4, iters=2000,
                                                        batch=8192, lr=1e-3, val_seeds=[15])
    ev = learned.evaluate(mlp, 21, 16, 8)
    assert npairs > 0 and np.isfinite(loss)
    assert ev["corrected_status"] == 0 and ev["corrected_divb"] <= 1e-4
    assert ev["corrected_l1"] < ev["coarse_l1"], ev
    mlp.close()


def test_grid_inference_equals_matrix_inference_on_a_ragged_grid():
    """The correction's in-grid inference (each row gathers its 3x3x3 stencil
    of feature records by padded cell index, the cell index split by
    host-computed multipliers) against the matrix inference on feature rows
    built on the host, on a periodic 20 x 12 x 24 grid: the hydro increments
    (zero-mean, times the output scale) and the face-B curl of the vector
    potential that one application adds agree with the host's to the BF16
    rounding of the features; a wrong gather would move them by O(1)."""
    nx, ny, nz = 20, 12, 24
    s = ics.orszag_tang_3d(nx, seed=3, ny0=ny, nz0=nz)
    prm = Params(nx, ny, nz, precision=FP32, tau=1e-3)
    ng = prm.nord // 2
    mlp = learned.MLP(learned.init_params(4) * 0.3)
    mean = np.array([0.2, 0.01, -0.01, 0.0, 0.5, 0.0, 0.0, 0.0], np.float32)
    std = np.array([0.1, 0.2, 0.2, 0.1, 0.3, 0.2, 0.2, 0.1], np.float32)
    scale = np.full(8, 1e-3, np.float32)
    mlp.set_norm(mean, std, scale)
    with MHDSolver(prm, s) as g:
        f0 = g.fetch()
        mlp.apply(g)
        f1 = g.fetch()
    U0, U1 = learned.conserved(f0, ng), learned.conserved(f1, ng)
    Un = (U0 - mean[:, None, None, None].astype(np.float64)) / std[:, None, None, None]
    cols = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.roll(Un, shift=(-dx, -dy, -dz), axis=(1, 2, 3))
                cols.append(sh.reshape(8, -1, order="F").T)
    x = np.zeros((nx * ny * nz, learned.FIN), dtype=np.float32)
    x[:, :216] = np.concatenate(cols, axis=1)
    y = mlp.forward(learned.bf16_bits(x)).astype(np.float64)  # [cells, 8], x fastest
    mlp.close()
    # hydro increments: zero-mean outputs times the scale
    dh = (y[:, :5] - y[:, :5].mean(axis=0)) * scale[:5]
    dU = (U1[:5] - U0[:5]).reshape(5, -1, order="F").T
    for q in range(5):
        ref = dh[:, q]
        assert np.abs(dU[:, q] - ref).max() <= 2e-2 * np.abs(ref).max() + 1e-7, q
    # face B: the curl of the edge means of the cell potentials A = y[5:8] * scale
    A = (y[:, 5:8] * scale[5:8]).T.reshape(3, nx, ny, nz, order="F")
    r = np.roll

    def edge(a, ax1, ax2):
        v = A[a]
        return 0.25 * (v + r(v, 1, ax1) + r(v, 1, ax2) + r(r(v, 1, ax1), 1, ax2))
    ex, ey, ez = edge(0, 1, 2), edge(1, 0, 2), edge(2, 0, 1)
    hx, hy, hz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    d = lambda e, ax, h: (r(e, -1, ax) - e) / h
    ref = {"bi": d(ez, 1, hy) - d(ey, 2, hz), "bj": d(ex, 2, hz) - d(ez, 0, hx), "bk": d(ey, 0, hx) - d(ex, 1, hy)}
    sl = (slice(ng, ng + nx), slice(ng, ng + ny), slice(ng, ng + nz))
    for k in ("bi", "bj", "bk"):
        got = f1[k][sl] - f0[k][sl]
        assert np.abs(got - ref[k]).max() <= 2e-2 * np.abs(ref[k]).max() + 1e-6, k
