"""numpy restatement of the slice-count MLP (12 -> 64 -> 64 -> 7, ReLU, softmax,
mean cross-entropy) in float64 - TEST INFRASTRUCTURE ONLY: the checker for the GPU
training kernels' gradients.  Parameter layout as in include/ccsdt.h:
W1[64][12] b1[64] W2[64][64] b2[64] W3[7][64] b3[7]."""
from __future__ import annotations

import numpy as np

IN, H, OUT = 12, 64, 7
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]


def unpack(p):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def loss_and_grad(p, X, y):
    P = unpack(p)
    X = np.asarray(X, np.float64)
    a1 = X @ P["W1"].T + P["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(a2, 0)
    z = h2 @ P["W3"].T + P["b3"]
    z = z - z.max(1, keepdims=True)
    pr = np.exp(z) / np.exp(z).sum(1, keepdims=True)
    n = len(y)
    loss = -np.log(pr[np.arange(n), y]).mean()
    dz = pr.copy()
    dz[np.arange(n), y] -= 1
    dz /= n
    g = {"W3": dz.T @ h2, "b3": dz.sum(0)}
    da2 = (dz @ P["W3"]) * (a2 > 0)
    g["W2"] = da2.T @ h1
    g["b2"] = da2.sum(0)
    da1 = (da2 @ P["W2"]) * (a1 > 0)
    g["W1"] = da1.T @ X
    g["b1"] = da1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SIZES])
