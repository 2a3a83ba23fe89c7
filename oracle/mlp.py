"""CPU oracle of the engine's cost-model network (TEST INFRASTRUCTURE ONLY).

Forward pass and mean-squared-error gradient of the MLP of
symboliclib_gb300/csrc/engine/costmodel.cu (inputs -> hidden -> hidden -> 1,
ReLU), in float64 numpy, from the same flattened parameter vector
(W1 in x h, b1, W2 h x h, b2, W3 h, b3)."""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, inputs: int, hidden: int):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + inputs * hidden].reshape(inputs, hidden); o += inputs * hidden
    b1 = p[o:o + hidden]; o += hidden
    W2 = p[o:o + hidden * hidden].reshape(hidden, hidden); o += hidden * hidden
    b2 = p[o:o + hidden]; o += hidden
    W3 = p[o:o + hidden].reshape(hidden, 1); o += hidden
    b3 = p[o:o + 1]; o += 1
    assert o == len(p)
    return W1, b1, W2, b2, W3, b3


def forward(p, X, inputs, hidden):
    W1, b1, W2, b2, W3, b3 = unpack(p, inputs, hidden)
    X = np.asarray(X, np.float64)
    h1 = np.maximum(X @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return (h2 @ W3 + b3)[:, 0], (X, h1, h2)


def gradient(p, X, y, inputs, hidden):
    W1, b1, W2, b2, W3, b3 = unpack(p, inputs, hidden)
    out, (X, h1, h2) = forward(p, X, inputs, hidden)
    n = len(y)
    d3 = 2.0 * (out - np.asarray(y, np.float64)) / n
    gW3 = h2.T @ d3[:, None]
    gb3 = np.array([d3.sum()])
    d2 = (d3[:, None] @ W3.T) * (h2 > 0)
    gW2 = h1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ W2.T) * (h1 > 0)
    gW1 = X.T @ d1
    gb1 = d1.sum(0)
    loss = float(np.mean((out - y) ** 2))
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3]), loss
