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


# ---------------------------------------------------------------------------------------------
# 3D gate inputs and labels (FP64 restatement of hos_3d_gate.cu).  Reference formulas: the
# non-DF WENO5-AO indicators and weights (src/reconstruction.cpp:161-360, epsilon 1e-10), the
# 3D characteristic basis (src/basic_function.cpp:994-1095), the frame rotations
# (Ydirection / Zdirection, :1208-1224).
# ---------------------------------------------------------------------------------------------
D5 = np.array([0.5 * 0.15 * 0.15, 0.15 * 0.85, 0.5 * 0.15 * 0.15, 0.85])


def _betas5(s):
    # about the centre value: the indicators depend on differences only
    s = np.asarray(s, dtype=np.float64) - s[2]
    wn2, wn1, w0, wp1, wp2 = s
    b0 = 13.0 / 12.0 * (wn2 - 2 * wn1 + w0) ** 2 + 0.25 * (wn2 - 4 * wn1 + 3 * w0) ** 2
    b1 = 13.0 / 12.0 * (wn1 - 2 * w0 + wp1) ** 2 + 0.25 * (wn1 - wp1) ** 2
    b2 = 13.0 / 12.0 * (w0 - 2 * wp1 + wp2) ** 2 + 0.25 * (3 * w0 - 4 * wp1 + wp2) ** 2
    b3 = (1.0 / 5040.0) * (231153 * w0 * w0 + 104963 * wn1 * wn1 + 6908 * wn2 * wn2 - 38947 * wn2 * wp1
                           + 104963 * wp1 * wp1 + wn1 * (-51001 * wn2 + 179098 * wp1 - 38947 * wp2)
                           - 3 * w0 * (99692 * wn1 - 22641 * wn2 + 99692 * wp1 - 22641 * wp2)
                           + 8209 * wn2 * wp2 - 51001 * wp1 * wp2 + 6908 * wp2 * wp2)
    b = np.array([b0, b1, b2, b3])
    tau = (abs(b3 - b0) + abs(b3 - b1) + abs(b3 - b2)) / 3.0
    return b, tau


def indicators5(s):
    """7 normalised indicators of a 5-cell stencil: betas / (sum + tau + 1e-10 c^2) padded to 6, tau"""
    s = np.asarray(s, dtype=np.float64)
    b, tau = _betas5(s)
    inv = 1.0 / (b.sum() + tau + 1e-10 * s[2] * s[2] + 1e-30)
    return np.concatenate([b * inv, [0.0, 0.0], [tau * inv]])


def _rotate(ax, w):
    if ax == 0:
        return w.copy()
    if ax == 1:
        return np.array([w[0], w[2], -w[1], w[3], w[4]])
    return np.array([w[0], w[3], w[2], -w[1], w[4]])


def _prim5(w, gamma):
    r = w[0]
    u, v, z = w[1] / r, w[2] / r, w[3] / r
    return np.array([r, u, v, z, (gamma - 1) * (w[4] - 0.5 * r * (u * u + v * v + z * z))])


def _left_eig5(pr, gamma):
    c = np.sqrt(gamma * pr[4] / pr[0])
    alfa = (gamma - 1) / (2 * c * c)
    u, v, w = pr[1], pr[2], pr[3]
    r = c / (gamma - 1)
    H = 0.5 * (u * u + v * v + w * w) + c * r
    return alfa * np.array([[H + r * (u - c), -(u + r), -v, -w, 1],
                            [4 * r * c - 2 * H, 2 * u, 2 * v, 2 * w, -2],
                            [-v / alfa, 0, 1 / alfa, 0, 0],
                            [-w / alfa, 0, 0, 1 / alfa, 0],
                            [H - r * (u + c), r - u, -v, -w, 1]])


def features3d(W, cell, ax, gamma=1.4):
    """16 gate inputs of cell (i, j, k) along axis ax from the AoS state W[nx, ny, nz, 5]"""
    i, j, k = cell
    st = []
    for m in range(-2, 3):
        idx = [i, j, k]
        idx[ax] += m
        st.append(W[tuple(idx)])
    rho = np.array([q[0] for q in st])
    p = np.array([(gamma - 1) * (q[4] - 0.5 * (q[1] ** 2 + q[2] ** 2 + q[3] ** 2) / q[0]) for q in st])
    return np.concatenate([indicators5(rho), indicators5(p), [0.0, 0.0]])


def distance3d(W, cell, ax, gamma=1.4, characteristic=True):
    """largest |omega_k - d_k| of the WENO5-AO weights over both faces and 5 variables"""
    i, j, k = cell
    st = []
    for m in range(-2, 3):
        idx = [i, j, k]
        idx[ax] += m
        st.append(_rotate(ax, W[tuple(idx)]))
    pr = [_prim5(st[m], gamma) for m in (1, 2, 3)]
    dmax = 0.0
    for side in (0, 1):
        base = 0.5 * ((pr[0] if side == 0 else pr[2]) + pr[1])
        L = _left_eig5(base, gamma) if characteristic else np.eye(5)
        ch = np.array([L @ q for q in st])      # [m][v]
        for v in range(5):
            b, tau = _betas5(ch[:, v])
            al = D5 * (1.0 + (tau / (b + 1e-6)) ** 2)
            dmax = max(dmax, float(np.abs(al / al.sum() - D5).max()))
    return dmax
