"""CPU check of the learned stencil classifier (test infrastructure): forward pass, mean binary
cross-entropy and its gradient for the 6 -> 32 -> 32 -> 3 MLP, in float64 with the same BF16
roundings the tensor-core kernels apply (weights, inputs, hidden activations and the
back-propagated error terms that feed the matrix products).  The classifier has no counterpart
in the reference; what it predicts is the reference's TENO5 cut-off (Schemes_Lagrange.cpp:
1141-1149), restated in oracle.hpp."""
from __future__ import annotations

import numpy as np

N_PARAMS = 192 + 32 + 1024 + 32 + 96 + 3


_EXACT = False


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64 (identity while
    exact(True) is in effect, for finite-difference checks of the formulas)."""
    if _EXACT:
        return np.asarray(a, dtype=np.float64)
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


class exact:
    """Context manager switching the BF16 roundings off."""

    def __init__(self, on=True):
        self.on = on

    def __enter__(self):
        global _EXACT
        self.prev, _EXACT = _EXACT, self.on

    def __exit__(self, *a):
        global _EXACT
        _EXACT = self.prev


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[0:192].reshape(32, 6)
    b1 = p[192:224]
    W2 = p[224:1248].reshape(32, 32)
    b2 = p[1248:1280]
    W3 = p[1280:1376].reshape(3, 32)
    b3 = p[1376:1379]
    return W1, b1, W2, b2, W3, b3


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def forward(p, x):
    """x: [n, 6] (already BF16 values).  Returns (z1, h1, z2, h2, z3) with BF16-rounded h."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    W1, W2, W3 = bf16(W1), bf16(W2), bf16(W3)
    z1 = x @ W1.T + b1
    h1 = bf16(np.maximum(z1, 0.0))
    z2 = h1 @ W2.T + b2
    h2 = bf16(np.maximum(z2, 0.0))
    z3 = h2 @ W3.T + b3
    return z1, h1, z2, h2, z3


def predict(p, x):
    return 1.0 / (1.0 + np.exp(-forward(p, x)[4]))


def loss_and_grad(p, x, labels):
    """Mean BCE over the rows and its gradient (parameter layout of hteno_mlp_get_params)."""
    n = x.shape[0]
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y = np.stack([(labels >> k) & 1 for k in range(3)], axis=1).astype(np.float64)
    z1, h1, z2, h2, z3 = forward(p, x)
    loss = (np.maximum(z3, 0) - z3 * y + np.log1p(np.exp(-np.abs(z3)))).sum() / n
    dz3 = bf16((1.0 / (1.0 + np.exp(-z3)) - y) / n)
    gW3 = dz3.T @ h2
    gb3 = dz3.sum(axis=0)
    dh2 = dz3 @ bf16(W3)
    dz2 = bf16(np.where(h2 > 0, dh2, 0.0))
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dh1 = dz2 @ bf16(W2)
    dz1 = bf16(np.where(h1 > 0, dh1, 0.0))
    gW1 = dz1.T @ x
    gb1 = dz1.sum(axis=0)
    return loss, pack(gW1, gb1, gW2, gb2, gW3, gb3)


def normalise(stencils):
    """(u - mean) / (max - min + 1e-30) per 6-cell row, clamped to [-1, 1]."""
    s = np.asarray(stencils, dtype=np.float64)
    v = (s - s.mean(axis=1, keepdims=True)) / (s.max(axis=1, keepdims=True) - s.min(axis=1, keepdims=True) + 1e-30)
    return np.clip(v, -1.0, 1.0)


def flat(stencils):
    """Rows whose six values are equal once rounded to float (not recorded by the harvest)."""
    f = np.asarray(stencils, dtype=np.float64).astype(np.float32)
    return (f == f[:, :1]).all(axis=1)
