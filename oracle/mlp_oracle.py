"""FP64 CPU restatement of the warm-start MLP (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: what the tests compare the device training and
inference kernels (ed_mlp_* in the library) against. It rounds to bfloat16 at
exactly the points where the device stores bfloat16 (input features, weights,
hidden activations, the gradients fed to the next matrix products) and
computes everything else in FP64, so device/oracle differences reduce to the
device's FP32 accumulation. The network has no reference counterpart (the
reference starts ARPACK from a random or file vector).
"""
from __future__ import annotations

import numpy as np

K_IN, K_OUT = 64, 8


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = x.view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    b = ((b + 0x7FFF + lsb) & 0xFFFF0000).astype(np.uint32)
    return b.view(np.float32).astype(np.float64)


def layout(norb: int, hidden: int):
    dims = [K_IN, hidden, hidden, hidden, K_OUT]
    offs = []
    off = 0
    for l in range(4):
        w = off
        off += dims[l] * dims[l + 1]
        b = off
        off += dims[l + 1]
        offs.append((w, b))
    return dims, offs, off


def unpack(p, norb, hidden):
    dims, offs, _ = layout(norb, hidden)
    Ws, bs = [], []
    for l, (w, b) in enumerate(offs):
        Ws.append(np.asarray(p[w:w + dims[l] * dims[l + 1]], dtype=np.float64).reshape(dims[l], dims[l + 1]))
        bs.append(np.asarray(p[b:b + dims[l + 1]], dtype=np.float64))
    return Ws, bs


def features(words, v1, norb):
    words = np.asarray(words, dtype=np.uint64)
    X = np.zeros((len(words), K_IN), dtype=np.float32)
    for k in range(norb):
        X[:, k] = np.where((words >> np.uint64(k)) & np.uint64(1), 1.0, -1.0)
    X[:, norb] = (np.asarray(v1, dtype=np.float32) - np.float32(1.75)) / np.float32(1.25)
    return bf16(X)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, words, v1, norb, hidden):
    Ws, bs = unpack(p, norb, hidden)
    x = features(words, v1, norb)
    Zs, Hs = [], [x]
    h = x
    for l in range(4):
        z = h @ bf16(Ws[l]) + bs[l]
        Zs.append(z)
        if l < 3:
            h = bf16(silu(z))
            Hs.append(h)
    return Zs, Hs


def loss_and_grads(p, words, v1, target, norb, hidden):
    """Loss mean[(y0 - t0)^2 + softplus(y1) - t1 y1] and its parameter gradient."""
    dims, offs, nparam = layout(norb, hidden)
    Ws, _ = unpack(p, norb, hidden)
    Zs, Hs = forward(p, words, v1, norb, hidden)
    m = len(words)
    y0, y1 = Zs[3][:, 0], Zs[3][:, 1]
    t0, t1 = target[:, 0].astype(np.float64), target[:, 1].astype(np.float64)
    loss = np.mean((y0 - t0) ** 2 + np.logaddexp(0.0, y1) - t1 * y1)
    dz = np.zeros((m, K_OUT))
    dz[:, 0] = 2.0 * (y0 - t0) / m
    dz[:, 1] = (1.0 / (1.0 + np.exp(-y1)) - t1) / m
    g = np.zeros(nparam)
    dzb = bf16(dz)
    for l in range(3, -1, -1):
        w, b = offs[l]
        g[w:w + dims[l] * dims[l + 1]] = (Hs[l].T @ dzb).ravel()
        g[b:b + dims[l + 1]] = dz.sum(axis=0)
        if l > 0:
            dh = dzb @ bf16(Ws[l]).T
            dz = dh * dsilu(Zs[l - 1])
            dzb = bf16(dz)
    return loss, g
