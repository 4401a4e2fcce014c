"""FP64 numpy restatement of the selector MLP (test infrastructure only).

Same architecture, parameter layout and loss as the library's CUDA kernels:
x -> standardise -> ReLU(W1 x + b1) -> ReLU(W2 h + b2) -> W3 h + b3, loss
sum(M * (Y - T)^2) / sum(M); parameters W1[h1,in], b1, W2[h2,h1], b2,
W3[out,h2], b3 packed in that order.  Used to check the library's gradients
and Adam updates.
"""
from __future__ import annotations

import numpy as np


def unpack(p, shape):
    i, h1, h2, o = shape
    sizes = [h1 * i, h1, h2 * h1, h2, o * h2, o]
    parts, k = [], 0
    for s in sizes:
        parts.append(p[k:k + s])
        k += s
    W1, b1, W2, b2, W3, b3 = parts
    return W1.reshape(h1, i), b1, W2.reshape(h2, h1), b2, W3.reshape(o, h2), b3


def num_params(shape):
    i, h1, h2, o = shape
    return h1 * i + h1 + h2 * h1 + h2 + o * h2 + o


def forward(p, shape, mean, std, X):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, np.float64), shape)
    Xn = (np.asarray(X, np.float64) - mean) / std
    A1 = np.maximum(Xn @ W1.T + b1, 0.0)
    A2 = np.maximum(A1 @ W2.T + b2, 0.0)
    return A2 @ W3.T + b3, (Xn, A1, A2)


def loss_and_grads(p, shape, mean, std, X, T, M):
    p = np.asarray(p, np.float64)
    Y, (Xn, A1, A2) = forward(p, shape, mean, std, X)
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    cnt = max(float(M.sum()), 1.0)
    D = Y - T
    loss = float((M * D * D).sum() / cnt)
    dY = 2.0 * M * D / cnt
    gW3 = dY.T @ A2
    gb3 = dY.sum(0)
    dA2 = (dY @ W3) * (A2 > 0)
    gW2 = dA2.T @ A1
    gb2 = dA2.sum(0)
    dA1 = (dA2 @ W2) * (A1 > 0)
    gW1 = dA1.T @ Xn
    gb1 = dA1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def loss_only(p, shape, mean, std, X, T, M):
    Y, _ = forward(p, shape, mean, std, X)
    cnt = max(float(M.sum()), 1.0)
    return float((M * (Y - T) ** 2).sum() / cnt)


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1 = 1 - b1 ** step
    c2 = 1 - b2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v
