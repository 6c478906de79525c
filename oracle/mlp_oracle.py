"""FP64 numpy reference of the warm-start MLP (TEST INFRASTRUCTURE ONLY).

Network 16 -> 128 -> 128 -> 128 -> 3 with SiLU after the hidden layers;
parameters flat as W1[128][16] b1 W2[128][128] b2 W3[128][128] b3 W4[3][128] b4.
Inputs normalised as (x - mean) / std, outputs multiplied by out_scale.
Loss: mean over rows of ||z4 - t / out_scale||^2 (z4 = normalised output).
The GPU kernels' gradients are checked against `loss_grad` here, and
`loss_grad` itself against central finite differences; `adam_update` restates the
optimiser the training kernels apply (Kingma & Ba 2015, bias-corrected
moments).
"""
from __future__ import annotations

import numpy as np

SIZES = [(16, 128), (128, 128), (128, 128), (128, 3)]


def unpack(p):
    out, off = [], 0
    for fi, fo in SIZES:
        W = p[off:off + fi * fo].reshape(fo, fi)
        off += fi * fo
        b = p[off:off + fo]
        off += fo
        out.append((W, b))
    return out


def n_params():
    return sum(fi * fo + fo for fi, fo in SIZES)


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(p, x, mean, std, scale):
    layers = unpack(np.asarray(p, np.float64))
    a = (np.asarray(x, np.float64) - mean) / std
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = silu(z) if l < 3 else z
    return a * scale


def loss_grad(p, x, t, mean, std, scale):
    layers = unpack(np.asarray(p, np.float64))
    n = len(x)
    acts = [(np.asarray(x, np.float64) - mean) / std]
    zs = []
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        zs.append(z)
        acts.append(silu(z) if l < 3 else z)
    d = acts[-1] - np.asarray(t, np.float64) / scale
    loss = float((d * d).sum() / n)
    dz = 2.0 * d / n
    grads = [None] * 4
    for l in range(3, -1, -1):
        W, _ = layers[l]
        grads[l] = (dz.T @ acts[l], dz.sum(0))
        if l == 0:
            break
        da = dz @ W
        s = 1.0 / (1.0 + np.exp(-zs[l - 1]))
        dz = da * s * (1.0 + zs[l - 1] * (1.0 - s))
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def adam_update(p, g, m, v, k: int, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
    """Adam step number k (from 1) with gradient g and moments m, v (zero
    before the first step): m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g^2,
    p - lr (m / (1 - b1^k)) / (sqrt(v / (1 - b2^k)) + eps).  Returns
    (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    return p - lr * (m / (1 - b1 ** k)) / (np.sqrt(v / (1 - b2 ** k)) + eps), m, v
