"""CPU oracle of the learned WENO gate's network -- test infrastructure only.

Restates, in numpy float64, the network the GPU kernels implement
(microfc_gb300/csrc/mfc_gate.cu, mfc_gate.cuh): inputs, the 10-32-32-1 ReLU
MLP, the weighted binary cross-entropy loss and its analytic gradient, plus
the FP16-weight / FP32-accumulate forward of the tensor-core inference.  The
analytic gradient is itself pinned by finite differences in the tests.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H = 10, 32
W1, B1 = 0, N_IN * N_H
W2 = B1 + N_H
B2 = W2 + N_H * N_H
W3 = B2 + N_H
B3 = W3 + N_H
N_PARAMS = B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(N_IN, N_H), p[B1:W2], p[W2:B2].reshape(N_H, N_H), p[B2:W3], p[W3:B3], p[B3])


def norm5(s, abs_floor):
    """(s - min) / max(max - min, 1e-2 * max|s|, abs_floor) for stencils s[..., 5]."""
    s = np.asarray(s, dtype=np.float64)
    lo, hi = s.min(axis=-1, keepdims=True), s.max(axis=-1, keepdims=True)
    fl = np.maximum(np.maximum(np.abs(lo), np.abs(hi)) * 1e-2, abs_floor)
    return (s - lo) / np.maximum(hi - lo, fl)


def features(alpha5, p5):
    return np.concatenate([norm5(alpha5, 1e-2), norm5(p5, 1e-30)], axis=-1)


def weight_deviation(x5, eps=1e-2):
    """max_k |omega_k - d_k| over both faces of the uniform-grid WENO5-JS
    weights of normalised stencils x5[..., 5] (the label statistic)."""
    v = [x5[..., k] for k in range(5)]
    b0 = 13 / 12 * (v[2] - 2 * v[3] + v[4]) ** 2 + 0.25 * (3 * v[2] - 4 * v[3] + v[4]) ** 2
    b1 = 13 / 12 * (v[1] - 2 * v[2] + v[3]) ** 2 + 0.25 * (v[1] - v[3]) ** 2
    b2 = 13 / 12 * (v[0] - 2 * v[1] + v[2]) ** 2 + 0.25 * (v[0] - 4 * v[1] + 3 * v[2]) ** 2
    out = np.zeros_like(b0)
    for d in ((0.1, 0.6, 0.3), (0.3, 0.6, 0.1)):  # left face, right face
        al = [d[k] / (b + eps) ** 2 for k, b in enumerate((b0, b1, b2))]
        s = al[0] + al[1] + al[2]
        for k in range(3):
            out = np.maximum(out, np.abs(al[k] / s - d[k]))
    return out


def forward(X, p):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    h1 = np.maximum(X @ w1 + b1, 0.0)
    h2 = np.maximum(h1 @ w2 + b2, 0.0)
    return h2 @ w3 + b3, (h1, h2)


def loss(X, t, p, pos_weight=1.0):
    z, _ = forward(X, p)
    sp_neg = np.logaddexp(0.0, -z)  # -log sigmoid(z)
    sp_pos = sp_neg + z             # -log(1 - sigmoid(z))
    return float(np.sum(pos_weight * t * sp_neg + (1.0 - t) * sp_pos))


def gradient(X, t, p, pos_weight=1.0):
    """Gradient of the MEAN loss over the batch (the kernels' convention)."""
    X = np.asarray(X, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    B = len(X)
    w1, b1, w2, b2, w3, b3 = unpack(p)
    z, (h1, h2) = forward(X, p)
    sig = 1.0 / (1.0 + np.exp(-z))
    dz = (sig * (pos_weight * t + 1.0 - t) - pos_weight * t) / B
    dh2 = np.outer(dz, w3) * (h2 > 0)
    dh1 = (dh2 @ w2.T) * (h1 > 0)
    g = np.zeros(N_PARAMS)
    g[W1:B1] = (X.T @ dh1).ravel()
    g[B1:W2] = dh1.sum(0)
    g[W2:B2] = (h1.T @ dh2).ravel()
    g[B2:W3] = dh2.sum(0)
    g[W3:B3] = h2.T @ dz
    g[B3] = dz.sum()
    return g


def forward_fp16(X, p):
    """FP16 inputs, weights and hidden activations, FP32 accumulation."""
    q = np.asarray(p, dtype=np.float32).astype(np.float16).astype(np.float32)
    w1, b1, w2, b2, w3, b3 = (a.astype(np.float32) for a in unpack(q))
    x = np.asarray(X, dtype=np.float32).astype(np.float16).astype(np.float32)
    h1 = np.maximum(x @ w1 + b1, 0).astype(np.float16).astype(np.float32)
    h2 = np.maximum(h1 @ w2 + b2, 0).astype(np.float16).astype(np.float32)
    return h2 @ w3 + np.float32(b3)
