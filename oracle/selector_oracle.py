"""CPU oracle for the precision-selector network (TEST INFRASTRUCTURE).

Only tests import this module.  It restates, in float64 numpy, the network
that uhm_gb300/csrc/k_selector.cu trains and runs on the device:

    h1 = relu(W1 x + b1)        W1: 64 x 12
    h2 = relu(W2 h1 + b2)       W2: 64 x 64
    z  = W3 h2 + b3             W3: 3 x 64
    loss = (1/B) sum_b w[y_b] * (logsumexp(z_b) - z_b[y_b])

with the parameters packed as W1, b1, W2, b2, W3, b3 (row-major), and its
exact gradient by backpropagation.  The selector has no counterpart in the
reference; this oracle is pinned by a finite-difference check in the tests.
"""
from __future__ import annotations

import numpy as np

F, H, C = 12, 64, 3
SHAPES = [(H, F), (H,), (H, H), (H,), (C, H), (C,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    out, o = [], 0
    for s in SHAPES:
        k = int(np.prod(s))
        out.append(p[o:o + k].reshape(s))
        o += k
    return out


def forward(params, X):
    W1, b1, W2, b2, W3, b3 = unpack(params)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ W3.T + b3
    return h1, h2, z


def loss_and_grad(params, X, y, class_weight=None):
    W1, b1, W2, b2, W3, b3 = unpack(params)
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.int64)
    B = X.shape[0]
    w = np.ones(C) if class_weight is None else np.asarray(class_weight, dtype=np.float64)
    h1, h2, z = forward(params, X)
    zm = z.max(axis=1, keepdims=True)
    lse = zm[:, 0] + np.log(np.exp(z - zm).sum(axis=1))
    wy = w[y]
    loss = float(np.sum(wy * (lse - z[np.arange(B), y])) / B)
    p = np.exp(z - lse[:, None])
    dz = p.copy()
    dz[np.arange(B), y] -= 1.0
    dz *= (wy / B)[:, None]
    dW3 = dz.T @ h2
    db3 = dz.sum(axis=0)
    dh2 = (dz @ W3) * (h2 > 0)
    dW2 = dh2.T @ h1
    db2 = dh2.sum(axis=0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    dW1 = dh1.T @ X
    db1 = dh1.sum(axis=0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return loss, g


def predict(params, X):
    _, _, z = forward(params, X)
    return z.argmax(axis=1)
