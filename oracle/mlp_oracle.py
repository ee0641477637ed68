"""ORACLE — test infrastructure only.

CPU restatement (numpy, float64) of the learned-shift MLP of the product library
(par_ilu0_cpp_gb300/csrc/mlp.cuh): the per-row features, the 4-16-16-1 network with
tanh hidden layers and a softplus output, the mean-squared-error loss and its gradient
by backpropagation.  Used only by tests, to check the GPU kernels' features, forward
pass and gradients.
"""
from __future__ import annotations

import numpy as np

IN, H = 4, 16
W1, B1 = 0, H * IN
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
NPARAMS = B3 + 1
DOMINANCE_CAP = 4.0


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(H, IN), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3], p[W3:B3], p[B3])


def features(a, depth=None, nlev=1):
    """Rows of [log(|a_ii|/mean|a_jj|), log(||a_i,off||_2/mean|a_jj|), min(dominance, 4), depth/(nlev-1)]."""
    n = a.n
    rows = np.repeat(np.arange(n), np.diff(a.row_ptr))
    isdiag = a.col_idx == rows
    absv = np.abs(a.values)
    d = np.zeros(n)
    d[rows[isdiag]] = absv[isdiag]
    offsum = np.bincount(rows[~isdiag], weights=absv[~isdiag], minlength=n)
    off2 = np.sqrt(np.bincount(rows[~isdiag], weights=a.values[~isdiag] ** 2, minlength=n))
    md = d.mean() if n else 1.0
    md = md if md > 0 else 1.0
    x0 = np.log(np.maximum(d, 1e-300) / md)
    x1 = np.log(np.maximum(off2, 1e-300) / md)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(offsum > 0, d / np.where(offsum > 0, offsum, 1.0), DOMINANCE_CAP)
    x2 = np.minimum(r, DOMINANCE_CAP)
    dep = np.zeros(n) if depth is None else np.asarray(depth, dtype=np.float64)
    x3 = dep / max(nlev - 1, 1)
    return np.stack([x0, x1, x2, x3], axis=1), offsum


def forward(p, X):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    h1 = np.tanh(X @ w1.T + b1)
    h2 = np.tanh(h1 @ w2.T + b2)
    z = h2 @ w3 + b3
    y = np.logaddexp(0.0, z)  # softplus
    return y, (h1, h2, z)


def loss_and_grad(p, X, T):
    """Mean squared error of softplus(MLP(X)) against T and its gradient (float64)."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    w1, b1, w2, b2, w3, b3 = unpack(p)
    y, (h1, h2, z) = forward(p, X)
    B = X.shape[0]
    diff = y - T
    loss = float(np.mean(diff ** 2))
    dz = 2.0 * diff / B / (1.0 + np.exp(-z))
    g = np.zeros(NPARAMS)
    g[B3] = dz.sum()
    g[W3:B3] = dz @ h2
    dh2 = np.outer(dz, w3) * (1.0 - h2 ** 2)
    g[B2:W3] = dh2.sum(axis=0)
    g[W2:B2] = (dh2.T @ h1).ravel()
    dh1 = (dh2 @ w2) * (1.0 - h1 ** 2)
    g[B1:W2] = dh1.sum(axis=0)
    g[W1:B1] = (dh1.T @ X).ravel()
    return loss, g
