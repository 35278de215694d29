"""ORACLE — test infrastructure only.

FP64 numpy restatement of the learned tuner's MLP (D -> 64 -> 64 -> 1,
ReLU; parameter layout W1[D][64] b1 W2[64][64] b2 W3[64] b3), its MSE loss
and Adam step, used to check the CUDA kernels' forward pass and gradients.
There is no reference implementation of this model; the restatement itself
is pinned by central finite differences (check_gradients_fd).
"""
from __future__ import annotations

import numpy as np

H = 64


def split(p, D):
    o = 0
    W1 = p[o:o + D * H].reshape(D, H); o += D * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(X, p, D):
    W1, b1, W2, b2, W3, b3 = split(np.asarray(p, dtype=np.float64), D)
    X = np.asarray(X, dtype=np.float64)
    A1 = np.maximum(X @ W1 + b1, 0.0)
    A2 = np.maximum(A1 @ W2 + b2, 0.0)
    Y = A2 @ W3 + b3
    return Y, A1, A2


def backward(X, p, D, dY):
    W1, b1, W2, b2, W3, b3 = split(np.asarray(p, dtype=np.float64), D)
    X = np.asarray(X, dtype=np.float64)
    dY = np.asarray(dY, dtype=np.float64)
    Y, A1, A2 = forward(X, p, D)
    dW3 = A2.T @ dY
    db3 = dY.sum()
    dZ2 = np.outer(dY, W3) * (A2 > 0)
    dW2 = A1.T @ dZ2
    db2 = dZ2.sum(0)
    dZ1 = (dZ2 @ W2.T) * (A1 > 0)
    dW1 = X.T @ dZ1
    db1 = dZ1.sum(0)
    return np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3, [db3]])


def mse(Y, T):
    e = np.asarray(Y, np.float64) - np.asarray(T, np.float64)
    return float((e * e).mean()), 2.0 * e / e.size


def check_gradients_fd(X, p, D, dY, idx, h=1e-6):
    """Central differences of L = sum(dY * Y) at the parameter indices idx."""
    g = backward(X, p, D, dY)
    out = []
    for i in idx:
        pp = np.array(p, dtype=np.float64)
        pp[i] += h
        lp = float(np.dot(dY, forward(X, pp, D)[0]))
        pp[i] -= 2 * h
        lm = float(np.dot(dY, forward(X, pp, D)[0]))
        out.append(((lp - lm) / (2 * h), g[i]))
    return out
