"""CPU oracle of the learned gate's network (test infrastructure only; never imported by the
product).  The gate has no counterpart in the reference: this is the repository's own
statement of it, used to check the GPU kernels.

The network is 16 -> 32 -> 32 -> 1 with ReLU; parameters are one float vector laid out as
W1[32][16], b1[32], W2[32][32], b2[32], w3[32], b3 (weights output-major).  With
``quantize=True`` the forward pass rounds the inputs, weights and hidden activations to
bfloat16 (round to nearest even) and accumulates in float32, as the tensor-core kernels do;
with ``quantize=False`` it runs in the dtype given (float64 for finite differences).  The loss
is the class-weighted mean binary cross-entropy of the logit against the label (1 = smooth).
"""
from __future__ import annotations

import numpy as np

NF, NH = 16, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAM = OFF_B3 + 1


def bf16(x) -> np.ndarray:
    """float32 -> bfloat16 -> float32 with round-to-nearest-even."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    return (p[OFF_W1:OFF_B1].reshape(NH, NF), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(NH, NH),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def forward(p, X, quantize=True):
    if quantize:
        q = bf16
        p = np.asarray(p, np.float32)
        X = np.asarray(X, np.float32)
    else:
        def q(a):
            return a
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = q(X)
    h1 = q(np.maximum(x @ q(W1).T + b1, 0))
    h2 = q(np.maximum(h1 @ q(W2).T + b2, 0))
    z = h2 @ q(w3) + b3
    return z, (x, h1, h2)


def loss_grad(p, X, y, w_pos=1.0, w_neg=4.0, quantize=True):
    """Mean weighted cross-entropy and its gradient with respect to the parameter vector (the
    gradient treats the bfloat16 roundings as identity, as the GPU backward pass does)."""
    z, (x, h1, h2) = forward(p, X, quantize)
    dt = z.dtype
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(p, dt))
    if quantize:
        W2, w3 = bf16(W2), bf16(w3)
    B = len(z)
    y = np.asarray(y) > 0.5
    sp = np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z)))
    loss = float(np.where(y, w_pos * (sp - z), w_neg * sp).sum() / B)
    pz = 1.0 / (1.0 + np.exp(-z))
    dz = (np.where(y, w_pos * (pz - 1.0), w_neg * pz) / B).astype(dt)
    d2 = np.where(h2 > 0, dz[:, None] * w3[None, :], 0).astype(dt)
    d1 = np.where(h1 > 0, d2 @ W2, 0).astype(dt)
    g = np.zeros(NPARAM, dt)
    g[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    g[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    g[OFF_W3:OFF_B3] = h2.T @ dz
    g[OFF_B3] = dz.sum()
    return loss, g


def finite_difference(p, X, y, idx, h=1e-6, w_pos=1.0, w_neg=4.0):
    """Central differences of the float64 loss for the parameters in idx."""
    p = np.asarray(p, np.float64).copy()
    out = []
    for k in idx:
        old = p[k]
        p[k] = old + h
        lp, _ = loss_grad(p, X, y, w_pos, w_neg, quantize=False)
        p[k] = old - h
        lm, _ = loss_grad(p, X, y, w_pos, w_neg, quantize=False)
        p[k] = old
        out.append((lp - lm) / (2 * h))
    return np.array(out)
