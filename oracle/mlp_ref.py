"""CPU restatement of the tuner network's forward pass and gradients.

TEST INFRASTRUCTURE ONLY: used by tests/ to check the CUDA training kernels
(race_gb300/csrc/mlp.cu) and never imported by the product.

The network has no counterpart in the reference (RACE tunes only by a
wall-clock sweep over powers, Interface::tuneFunction,
src/interface.cpp:605-647), so parity is pinned by mathematics instead of
golden vectors: the gradients below are checked against central finite
differences in float64 (tests/test_oracle.py), and the GPU gradients are
checked against these.

Layout (same as the CUDA side): layers l = 0..H, W_l row-major
[out_l][in_l] then b_l[out_l], flattened in that order; ReLU after every
layer except the last; loss = sum (y - t)^2 / (batch * out).
"""
from __future__ import annotations

import numpy as np


def shapes(n_in: int, hidden: int, hidden_layers: int, n_out: int):
    dims = [n_in] + [hidden] * hidden_layers + [n_out]
    return [(dims[l + 1], dims[l]) for l in range(len(dims) - 1)]


def num_params(n_in, hidden, hidden_layers, n_out) -> int:
    return sum(o * i + o for o, i in shapes(n_in, hidden, hidden_layers, n_out))


def unpack(theta, n_in, hidden, hidden_layers, n_out):
    out, off = [], 0
    for o, i in shapes(n_in, hidden, hidden_layers, n_out):
        W = theta[off: off + o * i].reshape(o, i)
        off += o * i
        b = theta[off: off + o]
        off += o
        out.append((W, b))
    return out


def forward(theta, X, dims):
    acts = [np.asarray(X, np.float64)]
    layers = unpack(np.asarray(theta, np.float64), *dims)
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        acts.append(z if l == len(layers) - 1 else np.maximum(z, 0.0))
    return acts


def loss_grad(theta, X, T, dims):
    """Loss and flat gradient (float64)."""
    acts = forward(theta, X, dims)
    layers = unpack(np.asarray(theta, np.float64), *dims)
    y = acts[-1]
    cnt = y.size
    d = 2.0 * (y - T) / cnt
    loss = float(np.sum((y - T) ** 2) / cnt)
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        xin = acts[l]
        grads[l] = (d.T @ xin, d.sum(axis=0))
        if l > 0:
            d = (d @ W) * (xin > 0)
    flat = np.concatenate([np.concatenate([gW.reshape(-1), gb]) for gW, gb in grads])
    return loss, flat

