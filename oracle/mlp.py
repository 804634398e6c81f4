"""Numpy restatement of the warm-start network (ORACLE, test infrastructure).

The network has no counterpart in the reference (whose EMI iteration starts from a
constant vector, phase_link/_eigenvalues.py:139-205): this module is the oracle for
the GPU kernels that train and run it.  A fully connected network with ReLU on the
hidden layers, weights W_l of shape (out, in), biases b_l, mean-squared-error loss
over all outputs, and Adam (Kingma & Ba 2015) with bias correction.
"""

from __future__ import annotations

import numpy as np

__all__ = ["adam_step", "backward", "bf16", "features", "forward", "forward_bf16", "mse"]


def features(C):
    """|C_ij| of the lower pairs (i > j, row by row) of (npix, n, n) coherence matrices."""
    C = np.asarray(C)
    n = C.shape[-1]
    i, j = np.tril_indices(n, -1)
    order = np.lexsort((j, i))  # row by row: (1,0), (2,0), (2,1), ...
    return np.abs(C[:, i[order], j[order]])


def forward(X, weights, biases):
    """Returns the list of layer outputs [H_1, ..., Y] (ReLU on all but the last)."""
    outs = []
    h = X
    for k, (W, b) in enumerate(zip(weights, biases)):
        z = h @ W.T + b
        h = np.maximum(z, 0) if k < len(weights) - 1 else z
        outs.append(h)
    return outs


def mse(Y, T):
    return float(np.mean((Y - T) ** 2))


def backward(X, T, weights, biases):
    """Gradients (dW_l, db_l) of mse(forward(X)[-1], T)."""
    outs = forward(X, weights, biases)
    Y = outs[-1]
    d = 2.0 * (Y - T) / Y.size
    gW, gb = [None] * len(weights), [None] * len(weights)
    for k in range(len(weights) - 1, -1, -1):
        h_in = X if k == 0 else outs[k - 1]
        gW[k] = d.T @ h_in
        gb[k] = d.sum(axis=0)
        if k > 0:
            d = (d @ weights[k]) * (outs[k - 1] > 0)
    return gW, gb


def adam_step(w, g, m, v, lr, b1, b2, eps, t):
    """One Adam update, in place on w, m, v."""
    m[...] = b1 * m + (1 - b1) * g
    v[...] = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1**t)
    vh = v / (1 - b2**t)
    w[...] = w - lr * mh / (np.sqrt(vh) + eps)


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward_bf16(X, weights, biases):
    """The output of a network whose inputs, weights and hidden activations are rounded
    to bfloat16, with exact (float64) accumulation and float32 biases: what a bf16
    tensor-core forward pass computes up to its fp32 accumulation order."""
    h = bf16(X).astype(np.float64)
    for k, (W, b) in enumerate(zip(weights, biases)):
        z = h @ bf16(W).astype(np.float64).T + np.asarray(b, np.float32)
        if k < len(weights) - 1:
            h = bf16(np.maximum(z, 0).astype(np.float32)).astype(np.float64)
        else:
            h = z
    return h
