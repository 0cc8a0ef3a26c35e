"""Numpy restatement of the corrector network's forward and backward passes — test infrastructure.

The network (femflow_gb300 learned corrector) is 128 (102 used) -> 64 -> 64 -> 64 -> 12 with GELU
between layers; it has no counterpart in the reference.  This oracle rounds to bfloat16 at exactly
the points where the GPU kernels store bf16 operands (weights, features, activations, output and
hidden gradients) and accumulates every product in float64, so it differs from the tensor-core
path only by the float32 accumulation order there.  Parameters use the flat layout of
include/femflow_mpm.h (FFMPM_MLP_OFF_*).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

OFF = {"W1": 0, "W2": 16384, "W3": 24576, "W4": 32768, "b1": 40960, "b2": 41024, "b3": 41088, "b4": 41152}
NPARAMS = 41168


def bf16(a) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    x = np.asarray(a, dtype=np.float32).copy()
    u = x.view(np.uint32)
    u += np.uint32(0x7FFF) + ((u >> np.uint32(16)) & np.uint32(1))
    u &= np.uint32(0xFFFF0000)
    return x.astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def _id(a):
    return np.asarray(a, dtype=np.float64)


def weights(P, rnd=bf16):
    P = np.asarray(P, dtype=np.float32 if rnd is bf16 else np.float64)
    W1 = P[OFF["W1"]:OFF["W1"] + 64 * 128].reshape(64, 128)
    W2 = P[OFF["W2"]:OFF["W2"] + 64 * 64].reshape(64, 64)
    W3 = P[OFF["W3"]:OFF["W3"] + 64 * 64].reshape(64, 64)
    W4 = P[OFF["W4"]:OFF["W4"] + 12 * 64].reshape(12, 64)
    b = [P[OFF[k]:OFF[k] + n].astype(np.float64) for k, n in (("b1", 64), ("b2", 64), ("b3", 64), ("b4", 12))]
    return [rnd(W) for W in (W1, W2, W3, W4)], b


def forward(P, X, exact=False):
    """X: scaled features as float values of bf16 [B][128].  Returns (Y [B][12], cache).
    exact=True: no bf16 rounding anywhere (float64 throughout)."""
    rnd = _id if exact else bf16
    (W1, W2, W3, W4), (b1, b2, b3, b4) = weights(P, rnd)
    X = np.asarray(X, dtype=np.float64)
    Z1 = X @ W1.T + b1
    H1 = rnd(gelu(Z1))
    Z2 = H1 @ W2.T + b2
    H2 = rnd(gelu(Z2))
    Z3 = H2 @ W3.T + b3
    H3 = rnd(gelu(Z3))
    Y = H3 @ W4.T + b4
    return Y, dict(X=X, Z1=Z1, H1=H1, Z2=Z2, H2=H2, Z3=Z3, H3=H3, W=(W1, W2, W3, W4))


def backward(P, X, T, w, exact=False):
    """Loss sum_j w_j (Y - T)^2 / B and its gradient in the flat parameter layout."""
    rnd = _id if exact else bf16
    f32 = (lambda a: a) if exact else (lambda a: a.astype(np.float32))
    Y, c = forward(P, X, exact)
    B = X.shape[0]
    w = np.asarray(w, dtype=np.float64)
    e = Y - T
    loss = float((w * e * e).sum() / B)
    g = np.zeros(NPARAMS)
    dY32 = f32(2.0 * w * e / B)
    dY = rnd(dY32)
    W1, W2, W3, W4 = c["W"]
    g[OFF["b4"]:OFF["b4"] + 12] = dY32.astype(np.float64).sum(axis=0)
    g[OFF["W4"]:OFF["W4"] + 12 * 64] = (dY.T @ c["H3"]).ravel()
    dZ3_32 = f32((dY @ W4) * gelu_grad(c["Z3"]))
    dZ3 = rnd(dZ3_32)
    g[OFF["b3"]:OFF["b3"] + 64] = dZ3_32.astype(np.float64).sum(axis=0)
    g[OFF["W3"]:OFF["W3"] + 64 * 64] = (dZ3.T @ c["H2"]).ravel()
    dZ2_32 = f32((dZ3 @ W3) * gelu_grad(c["Z2"]))
    dZ2 = rnd(dZ2_32)
    g[OFF["b2"]:OFF["b2"] + 64] = dZ2_32.astype(np.float64).sum(axis=0)
    g[OFF["W2"]:OFF["W2"] + 64 * 64] = (dZ2.T @ c["H1"]).ravel()
    dZ1_32 = f32((dZ2 @ W2) * gelu_grad(c["Z1"]))
    dZ1 = rnd(dZ1_32)
    g[OFF["b1"]:OFF["b1"] + 64] = dZ1_32.astype(np.float64).sum(axis=0)
    g[OFF["W1"]:OFF["W1"] + 64 * 128] = (dZ1.T @ c["X"]).ravel()
    return loss, g, Y


def forward_fp64(P, X):
    """The same network in float64 without any bf16 rounding (the ideal the bf16 path approximates)."""
    P = np.asarray(P, dtype=np.float64)
    W1 = P[OFF["W1"]:OFF["W1"] + 64 * 128].reshape(64, 128)
    W2 = P[OFF["W2"]:OFF["W2"] + 64 * 64].reshape(64, 64)
    W3 = P[OFF["W3"]:OFF["W3"] + 64 * 64].reshape(64, 64)
    W4 = P[OFF["W4"]:OFF["W4"] + 12 * 64].reshape(12, 64)
    b1, b2, b3, b4 = (P[OFF[k]:OFF[k] + n] for k, n in (("b1", 64), ("b2", 64), ("b3", 64), ("b4", 12)))
    H = gelu(np.asarray(X, dtype=np.float64) @ W1.T + b1)
    H = gelu(H @ W2.T + b2)
    H = gelu(H @ W3.T + b3)
    return H @ W4.T + b4
