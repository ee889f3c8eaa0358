"""ORACLE - test infrastructure only (tests/, smoke() and bench.py's
cpu_baseline leg). FP64 numpy restatement of the learned u_tau seed's
network and of its training gradient, against which the tests compare the
library's forward/backward kernels (include/foilcfd_wallnet.h).

The network has no counterpart in the reference (its wall model,
src/sim/lbm_wallmodel.cu:31-196, seeds Newton from the stored u_tau or
max(0.04 u, sqrt(nu u / y))). This restatement is pinned by its own
finite-difference check (gradient vs central differences of the forward, in
FP64) and, for the label solve, by the FP64 Newton of lbm_oracle.cpp, whose
root satisfies Reichardt's law to a relative residual below 1e-12.

Parameter layout (the library's): W1[32][3], b1[32], W2[32][32], b2[32],
W3[32], b3. Inputs x = (log u, log y, log nu - mean) * (1/std) with the
FP32 constants the kernels use; target t = (log u_tau - log u - out_mean) /
out_std; loss = mean (net(x) - t)^2.
"""
from __future__ import annotations

import numpy as np

H = 32
PARAMS = 1217


def unpack(p):
    p = np.asarray(p, np.float64)
    W1 = p[0:96].reshape(H, 3)
    b1 = p[96:128]
    W2 = p[128:1152].reshape(H, H)
    b2 = p[1152:1184]
    W3 = p[1184:1216]
    b3 = p[1216]
    return W1, b1, W2, b2, W3, b3


def bf16_round(p):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(p, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def inputs(norm, ut, ys, nu):
    """Normalised inputs with the kernels' FP32 constants (1/std in FP32)."""
    mean = np.asarray(norm["in_mean"], np.float32).astype(np.float64)
    inv = (np.float32(1.0) / np.asarray(norm["in_std"], np.float32)).astype(np.float64)
    x = np.stack([np.log(np.asarray(a, np.float64)) for a in (ut, ys, nu)], 1)
    return (x - mean) * inv


def target(norm, ut, tau):
    return (np.log(np.asarray(tau, np.float64)) - np.log(np.asarray(ut, np.float64)) - norm["out_mean"]) / norm["out_std"]


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3 + b3, (h1, h2)


def seed(p, norm, ut, ys, nu):
    """u_tau seed = u exp(out_mean + out_std net(x))."""
    y, _ = forward(p, inputs(norm, ut, ys, nu))
    return np.asarray(ut, np.float64) * np.exp(norm["out_mean"] + norm["out_std"] * y)


def loss_and_grad(p, x, t):
    """Mean squared error and its gradient w.r.t. the parameter vector."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = len(t)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    y = h2 @ W3 + b3
    err = y - t
    loss = np.mean(err ** 2)
    dy = 2.0 * err / n
    gW3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = (dy[:, None] * W3[None, :]) * (1 - h2 ** 2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (1 - h1 ** 2)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def finite_difference_grad(p, x, t, h=1e-6, idx=None):
    p = np.asarray(p, np.float64).copy()
    idx = range(PARAMS) if idx is None else idx
    out = {}
    for i in idx:
        old = p[i]
        p[i] = old + h
        lp = np.mean((forward(p, x)[0] - t) ** 2)
        p[i] = old - h
        lm = np.mean((forward(p, x)[0] - t) ** 2)
        p[i] = old
        out[i] = (lp - lm) / (2 * h)
    return out


def reference_seed(ut, ys, nu):
    """The reference's fresh seed max(0.04 u, sqrt(nu u / y)), FP32."""
    f = np.float32
    ut, ys, nu = (np.asarray(a, f) for a in (ut, ys, nu))
    return np.maximum(f(0.04) * ut, np.sqrt(nu * ut / ys)).astype(f)


def one_correction_residual(seed, ut, ys, nu):
    """FP32 emulation of the learned path's single Newton correction from
    `seed`: relative Reichardt residual |g| / u after it (accurate log1p/exp,
    as the kernel's library calls)."""
    f = np.float32
    K, C = f(0.41), f(7.8)
    ut, ys, nu = (np.asarray(a, f) for a in (ut, ys, nu))

    def reich(yp):
        e11 = np.exp(-yp / f(11)).astype(f)
        e3 = np.exp(-yp / f(3)).astype(f)
        up = (np.log1p(K * yp).astype(f) / K + C * (f(1) - e11 - (yp / f(11)) * e3)).astype(f)
        dup = (f(1) / (f(1) + K * yp) + C * ((f(1) / f(11)) * e11 - (f(1) / f(11)) * e3 + (yp / f(33)) * e3)).astype(f)
        return up, dup

    u = np.maximum(np.asarray(seed, f), f(1e-12))
    yp = (ys * u / nu).astype(f)
    up, dup = reich(yp)
    g = (u * up - ut).astype(f)
    u1 = np.maximum((u - g / np.maximum(up + yp * dup, f(1e-6))).astype(f), f(1e-12))
    yp = (ys * u1 / nu).astype(f)
    up, _ = reich(yp)
    return np.abs((u1 * up - ut).astype(f)).astype(np.float64) / ut
