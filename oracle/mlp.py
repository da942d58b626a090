"""CPU reference of the tuner network -- TEST INFRASTRUCTURE ONLY.

numpy forward and backward of the MLP that fastload_gb300/csrc/fl_mlp.cu
trains (ReLU hidden layers, linear output, masked mean-squared error), in
float64, with the same flat parameter order (W1, b1, W2, b2, W3, b3; W row-
major input x output).  Used to check the CUDA gradients."""
from __future__ import annotations

import numpy as np


def unpack(p, shape):
    i, h1, h2, o = shape
    sizes = [i * h1, h1, h1 * h2, h2, h2 * o, o]
    out, k = [], 0
    for s in sizes:
        out.append(np.asarray(p[k:k + s], np.float64))
        k += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(i, h1), b1, W2.reshape(h1, h2), b2, W3.reshape(h2, o), b3


def forward(p, shape, X):
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    X = np.asarray(X, np.float64)
    h1 = np.maximum(X @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h2 @ W3 + b3, (X, h1, h2)


def loss_grad(p, shape, X, T, M=None):
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    Y, (X, h1, h2) = forward(p, shape, X)
    T = np.asarray(T, np.float64)
    M = np.ones_like(T) if M is None else np.asarray(M, np.float64)
    cnt = M.sum()
    d = (Y - T) * M
    loss = float((d * d).sum() / cnt)
    dY = 2.0 * d / cnt
    dW3, db3 = h2.T @ dY, dY.sum(0)
    dh2 = (dY @ W3.T) * (h2 > 0)
    dW2, db2 = h1.T @ dh2, dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    dW1, db1 = X.T @ dh1, dh1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return loss, g
