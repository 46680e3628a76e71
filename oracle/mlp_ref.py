"""FP64 NumPy reference of the predictor MLP (TEST INFRASTRUCTURE ONLY): forward, MSE loss and
backward with the parameter layout of the CUDA network ([W1, b1, W2, b2, W3, b3], row-major,
y = W x + b per layer, exact GELU on the hidden layers).  Used to check the GPU gradients."""
from __future__ import annotations

import math

import numpy as np

_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_prime(z):
    cdf = 0.5 * (1.0 + _erf(z / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)
    return cdf + z * pdf


def unpack(p, shape):
    n_in, h1, h2, out = shape
    sizes = [h1 * n_in, h1, h2 * h1, h2, out * h2, out]
    parts, o = [], 0
    for s in sizes:
        parts.append(np.asarray(p[o:o + s], dtype=np.float64))
        o += s
    W1, b1, W2, b2, W3, b3 = parts
    return W1.reshape(h1, n_in), b1, W2.reshape(h2, h1), b2, W3.reshape(out, h2), b3


def forward(p, shape, X):
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    Z1 = X @ W1.T + b1
    H1 = gelu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = gelu(Z2)
    return H2 @ W3.T + b3, (Z1, H1, Z2, H2)


def loss_grad(p, shape, X, T):
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    Y, (Z1, H1, Z2, H2) = forward(p, shape, X)
    n = Y.size
    loss = 0.5 * np.sum((Y - T) ** 2) / n
    dY = (Y - T) / n
    gW3 = dY.T @ H2
    gb3 = dY.sum(0)
    dZ2 = (dY @ W3) * gelu_prime(Z2)
    gW2 = dZ2.T @ H1
    gb2 = dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * gelu_prime(Z1)
    gW1 = dZ1.T @ X
    gb1 = dZ1.sum(0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
