"""ORACLE -- test infrastructure only.  CPU (numpy) restatement of the learned
coarse-grid correction's network: forward pass, loss and backward pass of the
MLP 256 -> 64 -> 64 -> 16 (tanh-form GELU), in FP64 arithmetic.

With ``bf16=True`` it rounds the operands to BF16 exactly where the GPU
kernels do (features, weights, the hidden activations and the output and
hidden-layer gradients that feed a tensor-core GEMM), so that the GPU's FP32
accumulation is the only remaining difference; with ``bf16=False`` it is the
plain FP64 network, which tests check against finite differences.

Parameter layout (flat vector): W1[64][256] b1[64] W2[64][64] b2[64]
W3[16][64] b3[16]; inputs 216..255 and outputs 8..15 are padding.
"""
from __future__ import annotations

import numpy as np

FIN, NH, NO, NOUT = 256, 64, 16, 8
SHAPES = (("W1", (NH, FIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,)))
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p: np.ndarray) -> dict:
    out, off = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[off:off + n], dtype=np.float64).reshape(shape)
        off += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def bf16_bits(x) -> np.ndarray:
    """FP32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def bf16_val(bits) -> np.ndarray:
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def rb(x, on: bool) -> np.ndarray:
    """Round to BF16 (through FP32, as __float2bfloat16_rn does) when on."""
    return bf16_val(bf16_bits(np.asarray(x, dtype=np.float32))) if on else np.asarray(x, dtype=np.float64)


def gelu(z):
    c, a = np.sqrt(2.0 / np.pi), 0.044715
    t = np.tanh(c * (z + a * z ** 3))
    dg = 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * c * (1.0 + 3.0 * a * z * z)
    return 0.5 * z * (1.0 + t), dg


def init_params(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """He-style initialisation of the used part; padding rows/columns zero."""
    rng = np.random.default_rng(seed)
    d = {
        "W1": np.zeros((NH, FIN)), "b1": np.zeros(NH),
        "W2": rng.standard_normal((NH, NH)) * np.sqrt(2.0 / NH) * scale, "b2": np.zeros(NH),
        "W3": np.zeros((NO, NH)), "b3": np.zeros(NO),
    }
    d["W1"][:, :216] = rng.standard_normal((NH, 216)) * np.sqrt(2.0 / 216) * scale
    d["W3"][:NOUT] = rng.standard_normal((NOUT, NH)) * np.sqrt(1.0 / NH) * scale
    return pack(d).astype(np.float32)


def forward(p, x, bf16: bool = True) -> np.ndarray:
    """Raw outputs [n, 8] for features x [n, 256] (FP64 values)."""
    w = unpack(p)
    W1, W2, W3 = rb(w["W1"], bf16), rb(w["W2"], bf16), rb(w["W3"], bf16)
    z1 = x @ W1.T + w["b1"]
    h1 = rb(gelu(z1)[0], bf16)
    z2 = h1 @ W2.T + w["b2"]
    h2 = rb(gelu(z2)[0], bf16)
    return (h2 @ W3.T + w["b3"])[:, :NOUT]


def loss_and_grad(p, x, t, bf16: bool = True):
    """Mean squared error over samples and the 8 outputs, and its gradient
    (flat, parameter layout) in the GPU kernels' order of operations."""
    w = unpack(p)
    W1, W2, W3 = rb(w["W1"], bf16), rb(w["W2"], bf16), rb(w["W3"], bf16)
    n = x.shape[0]
    z1 = x @ W1.T + w["b1"]
    g1, dg1 = gelu(z1)
    h1 = rb(g1, bf16)
    z2 = h1 @ W2.T + w["b2"]
    g2, dg2 = gelu(z2)
    h2 = rb(g2, bf16)
    y = (h2 @ W3.T + w["b3"])[:, :NOUT]
    e = y - t
    loss = float(np.mean(e * e))
    dy = np.zeros((n, NO))
    dy[:, :NOUT] = 2.0 * e / (n * NOUT)
    dyb = rb(dy, bf16)
    gr = {"b3": dy.sum(0)}
    gr["W3"] = dyb.T @ h2
    dz2 = (dyb @ W3) * dg2
    dz2b = rb(dz2, bf16)
    gr["b2"] = dz2.sum(0)
    gr["W2"] = dz2b.T @ h1
    dz1 = (dz2b @ W2) * dg1
    dz1b = rb(dz1, bf16)
    gr["b1"] = dz1.sum(0)
    gr["W1"] = dz1b.T @ x
    return loss, pack(gr)
