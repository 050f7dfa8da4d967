"""Learned coarse-grid correction: data from the solver itself, training and
evaluation of the per-cell MLP whose training and inference kernels run on
the tensor cores (``csrc/mhd_mlp.cu``).

The network sees the 3x3x3 stencil of the 8 conserved variables (rho, rho v,
hydro energy, cell-centred B) of a coarse cell after a coarse step and
predicts 8 numbers: the increments of the 5 hydro conserved variables and a
cell-centred vector potential whose edge-averaged curl is added to the face
B, so the correction keeps div B at round-off.

Training pairs come from the solver: a fine 2N^3 run is restricted to N^3
(``restrict``: conservative 2x2x2 cell averages, face B as the mean of the 4
fine faces, which keeps div B = 0); the coarse solver takes one step of twice
the fine dt from the restriction at time t, and the target is the restriction
at t + 2 fine dt minus that coarse step.  The magnetic target is the vector
potential whose discrete curl (as the apply kernel computes it) best
reproduces the face-B difference (per-wavenumber least squares on the
periodic grid).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi, ics
from .abi import Params, FP32, STEP_RK2, check
from .solver import MHDSolver

FIN, NOUT = 256, 8
NPARAM = 64 * 256 + 64 + 64 * 64 + 64 + 16 * 64 + 16


def bf16_bits(x) -> np.ndarray:
    """FP32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


class MLP:
    """The network on the GPU (mhd_mlp_* entry points)."""

    def __init__(self, params: np.ndarray, lib=None):
        self.lib = lib or abi.load()
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == NPARAM
        h = C.c_void_p()
        check(self.lib, self.lib.mhd_mlp_create(p.ctypes.data, C.byref(h)), "mhd_mlp_create")
        self.h = h
        self.norm = None

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(NPARAM, dtype=np.float32)
        check(self.lib, self.lib.mhd_mlp_params(self.h, out.ctypes.data, None), "mhd_mlp_params")
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.lib, self.lib.mhd_mlp_params(self.h, None, p.ctypes.data), "mhd_mlp_params")

    def set_norm(self, mean, std, scale):
        a = [np.ascontiguousarray(v, dtype=np.float32) for v in (mean, std, scale)]
        check(self.lib, self.lib.mhd_mlp_set_norm(self.h, *[v.ctypes.data for v in a]), "mhd_mlp_set_norm")
        self.norm = a

    def set_data(self, xbits: np.ndarray, t: np.ndarray):
        xbits = np.ascontiguousarray(xbits, dtype=np.uint16)
        t = np.ascontiguousarray(t, dtype=np.float32)
        assert xbits.shape[1] == FIN and t.shape == (xbits.shape[0], NOUT)
        check(self.lib, self.lib.mhd_mlp_set_data(self.h, xbits.ctypes.data, t.ctypes.data, xbits.shape[0]),
              "mhd_mlp_set_data")

    def grad(self, offset: int, count: int):
        g = np.zeros(NPARAM, dtype=np.float32)
        loss = C.c_float()
        check(self.lib, self.lib.mhd_mlp_grad(self.h, int(offset), int(count), g.ctypes.data, C.byref(loss)),
              "mhd_mlp_grad")
        return loss.value, g

    def train(self, iters: int, batch: int = 16384, lr: float = 1e-3, seed: int = 0) -> float:
        loss = C.c_float()
        check(self.lib, self.lib.mhd_mlp_train(self.h, int(iters), int(batch), float(lr), int(seed), C.byref(loss)),
              "mhd_mlp_train")
        return loss.value

    def forward(self, xbits: np.ndarray) -> np.ndarray:
        xbits = np.ascontiguousarray(xbits, dtype=np.uint16)
        y = np.zeros((xbits.shape[0], NOUT), dtype=np.float32)
        check(self.lib, self.lib.mhd_mlp_forward(self.h, xbits.ctypes.data, xbits.shape[0], y.ctypes.data),
              "mhd_mlp_forward")
        return y

    def apply(self, solver: MHDSolver):
        check(self.lib, self.lib.mhd_mlp_apply(solver.h, self.h), "mhd_mlp_apply")

    def step_corrected(self, solver: MHDSolver, n: int):
        tau = C.c_double()
        st = C.c_uint32()
        check(self.lib, self.lib.mhd_step_corrected(solver.h, self.h, int(n), C.byref(tau), C.byref(st)),
              "mhd_step_corrected")
        return tau.value, st.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.mhd_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- host side
def conserved(f: dict, ng: int, gam: float = 5.0 / 3.0) -> np.ndarray:
    """U[8, nx0, ny0, nz0] of a fetched state: rho, rho v, hydro energy, cell B."""
    s = (slice(ng, -ng),) * 3
    r = f["rho"][s]
    u, v, w = f["vx"][s], f["vy"][s], f["vz"][s]
    e = 0.5 * r * (u * u + v * v + w * w) + f["p"][s] / (gam - 1.0)
    return np.stack([r, r * u, r * v, r * w, e, f["bx"][s], f["by"][s], f["bz"][s]])


def restrict(f: dict, n_fine: int, nord: int = 8, gam: float = 5.0 / 3.0) -> ics.State:
    """Coarse N^3 state (N = n_fine / 2) of a fine periodic state: 2x2x2 cell
    averages of the conserved variables, face B as the mean of the 4 fine
    faces covering each coarse face (div-free stays div-free)."""
    ng = nord // 2
    n = n_fine // 2
    U = conserved(f, ng, gam)
    Uc = U.reshape(8, n, 2, n, 2, n, 2).mean(axis=(2, 4, 6))
    s = ics.empty_state(ics.grid(n, n, n, nord=nord))
    sl = (slice(ng, ng + n),) * 3
    r = Uc[0]
    s.rho[sl] = r
    s.vx[sl], s.vy[sl], s.vz[sl] = Uc[1] / r, Uc[2] / r, Uc[3] / r
    s.p[sl] = (gam - 1.0) * (Uc[4] - 0.5 * (Uc[1] ** 2 + Uc[2] ** 2 + Uc[3] ** 2) / r)
    fi = f["bi"][ng:ng + n_fine, ng:ng + n_fine, ng:ng + n_fine]  # low faces of the fine interior cells
    fj = f["bj"][ng:ng + n_fine, ng:ng + n_fine, ng:ng + n_fine]
    fk = f["bk"][ng:ng + n_fine, ng:ng + n_fine, ng:ng + n_fine]
    bi = fi[0::2].reshape(n, n, 2, n, 2).mean(axis=(2, 4))
    bj = fj[:, 0::2].reshape(n, 2, n, n, 2).mean(axis=(1, 4))
    bk = fk[:, :, 0::2].reshape(n, 2, n, 2, n).mean(axis=(1, 3))
    ics._embed(s, {}, (bi, bj, bk))
    return s


def _faces(f: dict, ng: int, n: int):
    s = (slice(ng, ng + n),) * 3
    return f["bi"][s], f["bj"][s], f["bk"][s]


def curl_faces(A: np.ndarray, dx: float):
    """Face increments the apply kernel makes from cell-centred A[3, n, n, n]
    (periodic): edge potentials are 4-cell means, faces take their curl."""
    r = np.roll

    def edge(a, ax1, ax2):  # mean over the cells at -1 along ax1 and ax2
        v = A[a]
        return 0.25 * (v + r(v, 1, ax1) + r(v, 1, ax2) + r(r(v, 1, ax1), 1, ax2))
    ex, ey, ez = edge(0, 1, 2), edge(1, 0, 2), edge(2, 0, 1)
    d = lambda e, ax: (r(e, -1, ax) - e) / dx
    return d(ez, 1) - d(ey, 2), d(ex, 2) - d(ez, 0), d(ey, 0) - d(ex, 1)


_CURL_SVD = {}


def _curl_svd(n: int, dx: float):
    """Per-wavenumber SVD of the apply kernel's curl operator on an n^3
    periodic grid (cached: it depends on n and dx only)."""
    key = (n, dx)
    if key in _CURL_SVD:
        return _CURL_SVD[key]
    th = 2.0 * np.pi * np.fft.fftfreq(n)
    ex = np.exp(-1j * th)                      # shift by -1
    s = 0.5 * (1.0 + ex)                        # two-cell average toward -1
    dfw = (np.exp(1j * th) - 1.0) / dx          # forward difference
    S = [s[:, None, None], s[None, :, None], s[None, None, :]]
    D = [dfw[:, None, None], dfw[None, :, None], dfw[None, None, :]]
    shape = (n, n, n)
    M = np.zeros(shape + (3, 3), dtype=complex)
    # face_a += D_b E_c - D_c E_b with E_c = (avg over the two axes != c) A_c
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        M[..., a, c] = np.broadcast_to(D[b] * S[a] * S[b], shape)   # E_c averages over axes a, b
        M[..., a, b] = np.broadcast_to(-D[c] * S[a] * S[c], shape)  # E_b averages over axes c, a
    # minimum-norm solve; singular values below 1e-9 of the largest over all
    # wavenumbers are null directions (gauge, and the Nyquist modes that the
    # two-cell averages remove)
    u, sv, vh = np.linalg.svd(M)
    cut = 1e-9 * sv.max()
    inv = np.where(sv > cut, 1.0 / np.where(sv > cut, sv, 1.0), 0.0)
    _CURL_SVD.clear()  # keep one grid size
    _CURL_SVD[key] = (u, inv, vh)
    return u, inv, vh


def potential_from_faces(dbi, dbj, dbk, dx: float) -> np.ndarray:
    """Cell-centred A[3, n, n, n] whose edge-averaged discrete curl (the apply
    kernel's operator) is the least-squares fit of the face increments
    (periodic, per wavenumber, minimum-norm solution)."""
    n = dbi.shape[0]
    u, inv, vh = _curl_svd(n, dx)
    B = np.stack([np.fft.fftn(dbi), np.fft.fftn(dbj), np.fft.fftn(dbk)], axis=-1)
    uhb = np.einsum("...ji,...j->...i", u.conj(), B)
    A = np.einsum("...ji,...j->...i", vh.conj(), inv * uhb)
    return np.real(np.stack([np.fft.ifftn(A[..., i]) for i in range(3)]))


def features(U: np.ndarray, mean, std) -> np.ndarray:
    """BF16 feature rows [n^3, 256] (cell order x fastest) of periodic U[8, n, n, n]."""
    Un = (U - np.asarray(mean)[:, None, None, None]) / np.asarray(std)[:, None, None, None]
    n = U.shape[1]
    cols = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.roll(Un, shift=(-dx, -dy, -dz), axis=(1, 2, 3))
                cols.append(sh.reshape(8, -1, order="F").T)  # [cells, 8]
    x = np.zeros((n ** 3, FIN), dtype=np.float32)
    x[:, :216] = np.concatenate(cols, axis=1)
    return bf16_bits(x)


@dataclass
class Pairs:
    x: np.ndarray  # BF16 bits [m, 256]
    t: np.ndarray  # FP32 normalised targets [m, 8]


def generate(seeds, n_coarse: int, steps: int, every: int = 10, cfl: float = 0.3, nord: int = 8,
             norm=None, precision: int = FP32):
    """Training pairs from fine runs (2 n_coarse)^3 of the turbulence state,
    one snapshot every `every` fine steps; the fine runs in `precision` (the
    coarse step that the target corrects is FP32, as the corrected solver).
    Returns (raw features U list, raw targets list) for normalisation, then
    ``build`` packs them."""
    nf = 2 * n_coarse
    Us, Ts = [], []
    for seed in seeds:
        s = ics.turbulence(nf, seed=seed)
        tau_f = 0.8 * ics.cfl_dt(s, cfl=cfl)
        fine = MHDSolver(Params(nf, nf, nf, precision=precision, stepop=STEP_RK2, tau=tau_f, nord=nord), s)
        done = 0
        while done + 2 <= steps:
            f0 = fine.fetch()
            fine.step(2)
            f2 = fine.fetch()
            c0 = restrict(f0, nf, nord)
            tgt = restrict(f2, nf, nord)
            with MHDSolver(Params(n_coarse, n_coarse, n_coarse, precision=FP32, stepop=STEP_RK2, tau=2 * tau_f,
                                  nord=nord), c0) as cs:
                cs.step(1)
                c1 = cs.fetch()
            ng = nord // 2
            U1 = conserved(c1, ng)
            td = state_dict(tgt)
            Ut = conserved(td, ng)
            dB = [a - b for a, b in zip(_faces(td, ng, n_coarse), _faces(c1, ng, n_coarse))]
            A = potential_from_faces(*dB, dx=1.0 / n_coarse)
            Us.append(U1.astype(np.float32))
            Ts.append(np.concatenate([(Ut - U1)[:5], A]).astype(np.float32))
            fine.step(every - 2)
            done += every
        fine.close()
    return Us, Ts


def state_dict(s: ics.State) -> dict:
    """A State as the solver's fetch() dict, cell B as the face means (get_bxyz)."""
    d = {k: getattr(s, k) for k in ("rho", "vx", "vy", "vz", "p", "bi", "bj", "bk")}
    d["bx"] = 0.5 * (s.bi[1:] + s.bi[:-1])
    d["by"] = 0.5 * (s.bj[:, 1:] + s.bj[:, :-1])
    d["bz"] = 0.5 * (s.bk[:, :, 1:] + s.bk[:, :, :-1])
    return d


def normalisation(Us, Ts):
    """Per-variable feature mean/std and per-output target scales."""
    U = np.concatenate([u.reshape(8, -1) for u in Us], axis=1)
    T = np.concatenate([t.reshape(8, -1) for t in Ts], axis=1)
    mean, std = U.mean(1), U.std(1) + 1e-12
    scale = T.std(1) + 1e-30
    return mean.astype(np.float32), std.astype(np.float32), scale.astype(np.float32)


def build(Us, Ts, mean, std, scale, sample: float | None = None, seed: int = 0) -> Pairs:
    """Feature rows and normalised targets of every snapshot; with `sample`,
    a seeded random fraction of each snapshot's cells (bounds the pair count
    of large grids)."""
    rng = np.random.default_rng(seed)
    xs, ts = [], []
    for U, T in zip(Us, Ts):
        x = features(U, mean, std)
        t = (T.reshape(8, -1, order="F").T / scale).astype(np.float32)
        if sample is not None and sample < 1.0:
            keep = np.sort(rng.choice(x.shape[0], size=max(128, int(sample * x.shape[0])), replace=False))
            x, t = x[keep], t[keep]
        xs.append(x)
        ts.append(t)
    return Pairs(np.concatenate(xs), np.concatenate(ts))


def l1_error(a: dict, b: dict, ng: int) -> float:
    """Relative L1 error of the conserved variables of a against b (interior)."""
    Ua, Ub = conserved(a, ng), conserved(b, ng)
    return float(np.abs(Ua - Ub).sum() / np.abs(Ub).sum())


def evaluate(mlp: MLP, seed: int, n_coarse: int, steps: int, cfl: float = 0.3, nord: int = 8) -> dict:
    """Held-out comparison on one seed: the fine (2N)^3 run over 2*steps fine
    steps, restricted, is the reference; the plain and the corrected N^3 runs
    take `steps` steps of twice the fine dt.  Returns relative L1 errors of
    the conserved variables and the host wall time of each run (device
    synchronised at both ends)."""
    import time
    nf = 2 * n_coarse
    s = ics.turbulence(nf, seed=seed)
    tau_f = 0.8 * ics.cfl_dt(s, cfl=cfl)
    pf = Params(nf, nf, nf, precision=FP32, stepop=STEP_RK2, tau=tau_f, nord=nord)
    pc = Params(n_coarse, n_coarse, n_coarse, precision=FP32, stepop=STEP_RK2, tau=2 * tau_f, nord=nord)
    out = {}
    with MHDSolver(pf, s) as fine:
        c0 = restrict(fine.fetch(), nf, nord)
        fine.step(0)
        t0 = time.perf_counter()
        fine.step(2 * steps)
        out["fine_s"] = time.perf_counter() - t0
        ref = state_dict(restrict(fine.fetch(), nf, nord))
    ng = nord // 2
    with MHDSolver(pc, c0) as cs:
        cs.step(0)
        t0 = time.perf_counter()
        cs.step(steps)
        out["coarse_s"] = time.perf_counter() - t0
        out["coarse_l1"] = l1_error(cs.fetch(), ref, ng)
    with MHDSolver(pc, c0) as cs:
        cs.step(0)
        t0 = time.perf_counter()
        _, st = mlp.step_corrected(cs, steps)
        out["corrected_s"] = time.perf_counter() - t0
        f = cs.fetch()
        out["corrected_l1"] = l1_error(f, ref, ng)
        out["corrected_status"] = st
        out["corrected_divb"] = cs.diagnostics()["divb_max"]
    return out


# Dampings of the calibrated output strength tried by ``damp``.
DAMPINGS = (1.0, 0.75, 0.5, 0.25)


def choose_damping(error_of, gammas=DAMPINGS):
    """The damping gamma whose rollout error, error_of(gamma), is smallest.
    A correction trained on one-step residuals loses skill over a rollout as
    the coarse state drifts from the restricted fine states it learned from;
    damping its strength keeps most of the short-horizon skill at long
    horizons (CPU study, 16^3 coarse / 32^3 fine, FP64: x0.86 of the plain
    coarse error after 40 steps at gamma = 0.5, against x1.03 undamped).
    Returns (gamma, {gamma: error})."""
    errs = {float(g): float(error_of(g)) for g in gammas}
    return min(errs, key=errs.get), errs


def damp(mlp: MLP, seed: int, n_coarse: int, steps: int, gammas=DAMPINGS, nord: int = 8):
    """Choose the damping on a held-out seed's corrected rollout of `steps`
    coarse steps (``evaluate``) and leave the network's output scales at it.
    Returns (gamma, {gamma: corrected relative L1})."""
    mean, std, scale = mlp.norm

    def error_of(g):
        mlp.set_norm(mean, std, scale * np.float32(g))
        return evaluate(mlp, seed, n_coarse, steps, nord=nord)["corrected_l1"]

    g, errs = choose_damping(error_of, gammas)
    mlp.set_norm(mean, std, scale * np.float32(g))
    return g, errs


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initial weights of the used part; padding rows and columns zero."""
    rng = np.random.default_rng(seed)
    w1 = np.zeros((64, 256))
    w1[:, :216] = rng.standard_normal((64, 216)) * np.sqrt(2.0 / 216)
    w2 = rng.standard_normal((64, 64)) * np.sqrt(2.0 / 64)
    w3 = np.zeros((16, 64))
    w3[:8] = rng.standard_normal((8, 64)) * np.sqrt(1.0 / 64) * 0.1
    return np.concatenate([w1.ravel(), np.zeros(64), w2.ravel(), np.zeros(64), w3.ravel(),
                           np.zeros(16)]).astype(np.float32)


def calibrate(mlp: MLP, Us, Ts, mean, std, scale) -> np.ndarray:
    """Per-output least-squares shrinkage of the trained network on held-out
    pairs: alpha_q = <y_q, t_q> / <y_q, y_q>, clipped to [0, 1].  An output
    without skill on unseen data (alpha near 0) is switched off rather than
    allowed to add error.  Returns alpha; the network's output scales become
    scale * alpha."""
    num = np.zeros(8)
    den = np.zeros(8)
    for U, T in zip(Us, Ts):
        y = mlp.forward(features(U, mean, std)).astype(np.float64)
        t = T.reshape(8, -1, order="F").T / scale
        num += (y * t).sum(0)
        den += (y * y).sum(0)
    alpha = np.clip(num / np.maximum(den, 1e-30), 0.0, 1.0)
    mlp.set_norm(mean, std, (scale * alpha).astype(np.float32))
    return alpha


def train_correction(train_seeds, n_coarse: int, steps: int, every: int = 10, iters: int = 2000,
                     batch: int = 16384, lr: float = 1e-3, init_seed: int = 0, nord: int = 8,
                     val_seeds=None, sample: float | None = None, val_steps: int | None = None):
    """Generate pairs from the fine runs of train_seeds, normalise, train a
    fresh network and, with val_seeds, calibrate its outputs on their pairs.
    Returns (mlp, final minibatch loss, number of training pairs, alpha)."""
    Us, Ts = generate(train_seeds, n_coarse, steps, every=every, nord=nord)
    mean, std, scale = normalisation(Us, Ts)
    pairs = build(Us, Ts, mean, std, scale, sample=sample, seed=init_seed)
    del Us, Ts
    mlp = MLP(init_params(init_seed))
    mlp.set_norm(mean, std, scale)
    mlp.set_data(pairs.x, pairs.t)
    loss = mlp.train(iters, batch=min(batch, (pairs.x.shape[0] // 128) * 128), lr=lr, seed=init_seed)
    alpha = np.ones(8)
    if val_seeds:
        Uv, Tv = generate(val_seeds, n_coarse, val_steps or steps, every=every, nord=nord)
        alpha = calibrate(mlp, Uv, Tv, mean, std, scale)
    return mlp, loss, pairs.x.shape[0], alpha


def truth_compare(mlp: MLP, seed: int, n_coarse: int, steps: int, cfl: float = 0.3, nord: int = 8) -> dict:
    """Errors against a 4x finer truth: the (4N)^3 FP32 run over 4*steps steps,
    restricted to N^3, judges the plain (2N)^3 FP64 run (2*steps steps from
    the restricted truth start), the plain N^3 FP32 run and the corrected N^3
    run (steps steps).  GPU time: CUDA events around graph replays for the
    plain runs, host wall clock (device synchronised) for the corrected run."""
    import time
    n4, n2 = 4 * n_coarse, 2 * n_coarse
    s4 = ics.turbulence(n4, seed=seed)
    tau4 = 0.8 * ics.cfl_dt(s4, cfl=cfl)
    ng = nord // 2
    out = {}

    def timed(prm, st, k, chunk):
        with MHDSolver(prm, st) as sv:
            ms, done = 0.0, 0
            while done < k:
                m = min(chunk, k - done)
                ms += sv.time_steps(m, graph=True)
                done += m
            return ms, sv.fetch()

    ms4, f4 = timed(Params(n4, n4, n4, precision=FP32, stepop=STEP_RK2, tau=tau4, nord=nord), s4, 4 * steps, 100)
    ref = state_dict(restrict(state_dict(restrict(f4, n4, nord)), n2, nord))
    del f4
    with MHDSolver(Params(n4, n4, n4, precision=FP32, stepop=STEP_RK2, tau=tau4, nord=nord), s4) as sv:
        s2 = restrict(sv.fetch(), n4, nord)
    del s4
    s1 = restrict(state_dict(s2), n2, nord)
    from .abi import FP64
    ms2, f2 = timed(Params(n2, n2, n2, precision=FP64, stepop=STEP_RK2, tau=2 * tau4, nord=nord), s2, 2 * steps, 20)
    out["fine_fp64"] = {"n": n2, "steps": 2 * steps, "gpu_ms": ms2,
                        "l1": l1_error(state_dict(restrict(f2, n2, nord)), ref, ng)}
    del f2
    pc = Params(n_coarse, n_coarse, n_coarse, precision=FP32, stepop=STEP_RK2, tau=4 * tau4, nord=nord)
    ms1, f1 = timed(pc, s1, steps, 100)
    out["coarse_fp32"] = {"n": n_coarse, "steps": steps, "gpu_ms": ms1, "l1": l1_error(f1, ref, ng)}
    with MHDSolver(pc, s1) as cs:
        cs.step(0)
        t0 = time.perf_counter()
        _, st = mlp.step_corrected(cs, steps)
        t1 = time.perf_counter()
        out["corrected_fp32"] = {"n": n_coarse, "steps": steps, "wall_ms": 1e3 * (t1 - t0),
                                 "l1": l1_error(cs.fetch(), ref, ng), "status": st,
                                 "divb_max": cs.diagnostics()["divb_max"]}
    out["truth"] = {"n": n4, "steps": 4 * steps, "gpu_ms": ms4, "precision": "fp32"}
    return out
