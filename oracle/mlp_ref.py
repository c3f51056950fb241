"""FP64 numpy restatement of the bandwidth MLP -- TEST INFRASTRUCTURE ONLY.

Used by tests/ to check the gradients and outputs of the CUDA MLP kernels.
The network is 32 -> 128 -> 128 -> 3 with ReLU; the flat parameter layout is
[W1 (128x32), b1, W2 (128x128), b2, W3 (3x128), b3]. The CUDA passes use the
weights rounded to BF16 (biases stay FP32) on inputs normalised as
(x - mu) / sd and clipped to [-6, 6], so this reference does the same, in
FP64 otherwise. Loss:
sum(mask (y - t)^2) / sum(mask). Also restates the 32 summary features.
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 32, 128, 3
SHAPES = [("W1", (NH, NI)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
          ("W3", (NO, NH)), ("b3", (NO,))]


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([d[name].ravel() for name, _ in SHAPES])


def forward(p, mu, sd, X):
    w = unpack(np.asarray(p, np.float32))
    W1, W2, W3 = (bf16(w[k]).astype(np.float64) for k in ("W1", "W2", "W3"))
    b1, b2, b3 = (w[k].astype(np.float64) for k in ("b1", "b2", "b3"))
    x = (np.asarray(X, np.float32) - mu) / sd
    x = np.clip(x.astype(np.float32), -6.0, 6.0).astype(np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    y = h2 @ W3.T + b3
    return x, h1, h2, y, (W1, W2, W3)


def loss_and_grad(p, mu, sd, X, T, M):
    x, h1, h2, y, (W1, W2, W3) = forward(p, mu, sd, X)
    m = np.asarray(M, np.float64)
    ms = max(m.sum(), 1.0)
    e = y - np.asarray(T, np.float64)
    loss = float((m * e * e).sum() / ms)
    dy = 2 * m * e / ms
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    dh2 = (dy @ W3) * (h2 > 0)
    g["W2"], g["b2"] = dh2.T @ h1, dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    g["W1"], g["b1"] = dh1.T @ x, dh1.sum(0)
    return loss, pack(g)


def features(x: np.ndarray) -> np.ndarray:
    """The 32 features of one instance x (d, n), in FP64."""
    x = np.atleast_2d(np.asarray(x, np.float64))
    d, n = x.shape
    f = np.zeros(NI)
    for j in range(d):
        v = x[j]
        mean = v.mean()
        c = v - mean
        var = (c * c).mean()
        sd = np.sqrt(var)
        f[6 * j + 0] = mean
        f[6 * j + 1] = sd
        f[6 * j + 2] = (c ** 3).mean() / sd ** 3
        f[6 * j + 3] = (c ** 4).mean() / var ** 2 - 3
        s = np.sort(v.astype(np.float32)).astype(np.float64)
        # distance to the 8th nearest neighbour along the sorted order
        pad = np.concatenate([np.full(8, -np.inf), s, np.full(8, np.inf)])
        cand = np.stack([np.abs(pad[8 + k:8 + k + n] - s) for k in range(-8, 9) if k != 0])
        dk = np.sort(cand, axis=0)[7]
        f[6 * j + 4] = dk.mean() / sd
        f[6 * j + 5] = dk.std() / sd
        if j == 0:
            for q in range(1, 10):
                f[18 + q - 1] = (s[(q * (n - 1)) // 10] - mean) / sd
    f[27] = np.log(n)
    f[28] = d
    f[29:29 + d] = 1
    return f
