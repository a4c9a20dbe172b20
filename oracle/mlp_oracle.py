"""numpy restatement of the learned tuner's network (test infrastructure): the same
I -> H -> H -> K ReLU network, softmax and mean soft cross-entropy, with its analytic gradient.
The GPU kernels' gradients are checked against this, and this against finite differences."""
from __future__ import annotations

import numpy as np


def unpack(params: np.ndarray, I: int, H: int, K: int):
    p = np.asarray(params, np.float64)
    o = 0
    W1 = p[o:o + H * I].reshape(H, I); o += H * I
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + K * H].reshape(K, H); o += K * H
    b3 = p[o:o + K]; o += K
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(params, feats, mean, std, I, H, K):
    W1, b1, W2, b2, W3, b3 = unpack(params, I, H, K)
    xn = (np.asarray(feats, np.float64) - mean) / std
    z1 = xn @ W1.T + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0)
    z3 = a2 @ W3.T + b3
    z = z3 - z3.max(axis=1, keepdims=True)
    p = np.exp(z) / np.exp(z).sum(axis=1, keepdims=True)
    return dict(xn=xn, z1=z1, a1=a1, z2=z2, a2=a2, z3=z3, p=p)


def loss_and_grad(params, feats, targets, mean, std, I, H, K):
    W1, b1, W2, b2, W3, b3 = unpack(params, I, H, K)
    f = forward(params, feats, mean, std, I, H, K)
    B = f["p"].shape[0]
    t = np.asarray(targets, np.float64)
    logp = np.log(np.maximum(f["p"], 1e-300))
    loss = float(-(t * logp).sum() / B)
    dz3 = (f["p"] - t) / B
    gW3 = dz3.T @ f["a2"]
    gb3 = dz3.sum(0)
    dz2 = (dz3 @ W3) * (f["z2"] > 0)
    gW2 = dz2.T @ f["a1"]
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (f["z1"] > 0)
    gW1 = dz1.T @ f["xn"]
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
