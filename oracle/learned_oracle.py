"""FP64 numpy restatement of the learned row filter (TEST INFRASTRUCTURE ONLY).

Checks the library's CUDA forward/backward kernels (csrc/sgb_learned.cu): the network is
5 conv1d layers (kernel 9, zero padding 4; channels 1->32->32->32->32->1) with exact
(erf) GELU after the first four, applied as a residual y = z + s * net(z / s).  The loss
is mean((y - target)^2) / s^2.  Parameters are laid out layer by layer: W (cout, cin, 9)
then b (cout).  There is no reference counterpart (Sinograms.jl has no learned filter).
"""
from __future__ import annotations

import math

import numpy as np

K, PAD, C = 9, 4, 32
CIN = [1, C, C, C, C]
COUT = [C, C, C, C, 1]


def unpack(p: np.ndarray):
    out, o = [], 0
    for ci, co in zip(CIN, COUT):
        w = p[o:o + co * ci * K].reshape(co, ci, K)
        o += co * ci * K
        b = p[o:o + co]
        o += co
        out.append((w, b))
    assert o == p.size
    return out


def nparams() -> int:
    return sum(co * ci * K + co for ci, co in zip(CIN, COUT))


def _erf(x):
    from scipy.special import erf
    return erf(x)


def gelu(x):
    return 0.5 * x * (1 + _erf(x / math.sqrt(2)))


def gelu_grad(x):
    return 0.5 * (1 + _erf(x / math.sqrt(2))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def conv(x, w, b):
    """x (R, cin, L), w (cout, cin, K) -> (R, cout, L): y[t] = b + sum w[k] x[t+k-4]."""
    R, ci, L = x.shape
    xp = np.zeros((R, ci, L + 2 * PAD))
    xp[:, :, PAD:PAD + L] = x
    cols = np.stack([xp[:, :, k:k + L] for k in range(K)], axis=-1)  # (R, cin, L, K)
    return np.einsum("rclk,ock->rol", cols, w) + b[None, :, None]


def forward(p, z, scale, bf16_weights=True):
    """Returns (y, cache).  bf16_weights rounds W to bfloat16 as the GPU's forward does."""
    layers = unpack(np.asarray(p, np.float64))
    if bf16_weights:
        layers = [(_bf16(w), b) for w, b in layers]
    a = (np.asarray(z, np.float64) / scale)[:, None, :]
    acts, pres = [a], []
    for i, (w, b) in enumerate(layers):
        h = conv(a, w, b)
        if i < len(layers) - 1:
            pres.append(h)
            a = gelu(h)
        else:
            a = h
        acts.append(a)
    y = np.asarray(z, np.float64) + scale * a[:, 0, :]
    return y, (layers, acts, pres)


def loss_grad(p, z, target, scale, bf16_weights=True):
    """(loss, dloss/dp) with loss = mean((y - target)^2) / scale^2."""
    y, (layers, acts, pres) = forward(p, z, scale, bf16_weights)
    n = y.size
    d = (y - target) / scale
    loss = float(np.mean(d * d))
    g = (2 * d / n)[:, None, :]  # dloss/d(net output)
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        w, _ = layers[i]
        x = acts[i]
        R, ci, L = x.shape
        xp = np.zeros((R, ci, L + 2 * PAD))
        xp[:, :, PAD:PAD + L] = x
        cols = np.stack([xp[:, :, k:k + L] for k in range(K)], axis=-1)
        gw = np.einsum("rol,rclk->ock", g, cols)
        gb = g.sum(axis=(0, 2))
        grads[i] = (gw, gb)
        if i > 0:
            # dx[t] = sum_k w[k] g[t - k + 4]
            gp = np.zeros((R, g.shape[1], L + 2 * PAD))
            gp[:, :, PAD:PAD + L] = g
            gcols = np.stack([gp[:, :, 2 * PAD - k:2 * PAD - k + L] for k in range(K)], axis=-1)
            gx = np.einsum("rolk,ock->rcl", gcols, w)
            g = gx * gelu_grad(pres[i - 1])
    flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
    return loss, flat


def _bf16(w):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(w, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)
