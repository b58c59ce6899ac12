"""CPU oracle of the plan cost model's MLP (test infrastructure only).

The same network as the library's CUDA kernels (chfft_gb300/csrc/costmodel.cu):
f(x) = W3 relu(W2 relu(W1 x + b1) + b2) + b3 on standardised rows, loss
0.5 * mean((f(x) - y)^2), parameters flattened as W1 (H x F), b1, W2 (H x H),
b2, W3 (H), b3. Computed in float64 with numpy, so it checks the GPU
gradients; its own gradient is checked by finite differences. The network
has no counterpart in chfft.
"""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, f: int, h: int):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + h * f].reshape(h, f); o += h * f
    b1 = p[o:o + h]; o += h
    W2 = p[o:o + h * h].reshape(h, h); o += h * h
    b2 = p[o:o + h]; o += h
    W3 = p[o:o + h]; o += h
    b3 = p[o]; o += 1
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(p, X, f: int, h: int):
    W1, b1, W2, b2, W3, b3 = unpack(p, f, h)
    X = np.asarray(X, np.float64)
    a1 = np.maximum(X @ W1.T + b1, 0.0)
    a2 = np.maximum(a1 @ W2.T + b2, 0.0)
    return a2 @ W3 + b3


def loss_grad(p, X, y, f: int, h: int):
    """0.5 * mean((f(X) - y)^2) and its gradient in the flat parameter layout."""
    W1, b1, W2, b2, W3, b3 = unpack(p, f, h)
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    n = len(y)
    z1 = X @ W1.T + b1
    a1 = np.maximum(z1, 0.0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0.0)
    out = a2 @ W3 + b3
    r = out - y
    loss = 0.5 * np.mean(r * r)
    e = r / n
    gW3 = a2.T @ e
    gb3 = e.sum()
    d2 = np.outer(e, W3) * (z2 > 0)
    gW2 = d2.T @ a1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (z1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def standardise(X, y, mean, sd, y_mean, y_sd):
    return (np.asarray(X, np.float64) - mean) / sd, (np.asarray(y, np.float64) - y_mean) / y_sd
