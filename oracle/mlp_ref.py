"""CPU oracle of the chemistry surrogate's MLP: forward pass, mean-square
loss and backward pass in float64 NumPy.

Test infrastructure only: the GPU tests compare the library's tensor-core
forward/backward kernels with these functions on the same (BF16-rounded)
weights and inputs. It is pinned by central finite differences of its own
loss (tests/test_oracle_mlp.py). The reference code has no surrogate, so
this restates the standard MLP algebra:

    z_l = h_l W_l^T + b_l,  h_{l+1} = gelu(z_l)   (hidden layers)
    y   = h_L W_L^T + b_L
    loss = mean over rows and the first n_real columns of (y - t)^2
    gelu(z) = z Phi(z) = 0.5 z (1 + erf(z / sqrt 2))
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def dgelu(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(Ws, bs, X):
    """Returns (y, zs, hs): the output, the hidden pre-activations and the
    layer inputs (hs[0] = X)."""
    hs, zs = [X], []
    h = X
    for W, b in zip(Ws[:-1], bs[:-1]):
        z = h @ W.T + b
        zs.append(z)
        h = gelu(z)
        hs.append(h)
    y = h @ Ws[-1].T + bs[-1]
    return y, zs, hs


def loss_and_grads(Ws, bs, X, T, n_real):
    """Mean-square loss over the first n_real output columns and its
    gradients with respect to every W_l and b_l."""
    y, zs, hs = forward(Ws, bs, X)
    M = X.shape[0]
    d = np.zeros_like(y)
    d[:, :n_real] = y[:, :n_real] - T[:, :n_real]
    loss = float((d ** 2).sum() / (M * n_real))
    g = 2.0 * d / (M * n_real)
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        gW[l] = g.T @ hs[l]
        gb[l] = g.sum(axis=0)
        if l > 0:
            g = (g @ Ws[l]) * dgelu(zs[l - 1])
    return loss, gW, gb
