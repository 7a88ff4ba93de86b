"""FP64 restatement of the learned scheduler's MLP -- TEST INFRASTRUCTURE ONLY.

Forward pass, loss and gradients of the 4 -> 32 -> 32 -> 1 ReLU network in
numpy float64, with the parameter layout of the GPU kernels
(hsmu-spgemm_gb300/csrc/learned.cu): W1[32][4] b1[32] W2[32][32] b2[32]
W3[32] b3, then the normalisation constants mu[4] sd[4] ymu ysd.  Tests use
it to check the FP32 forward/gradient kernels; nothing in the engine calls it.
"""
from __future__ import annotations

import numpy as np

H, NF = 32, 4
O_W1, O_B1 = 0, H * NF
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + H
NPARAM = O_B3 + 1
O_MU, O_SD = NPARAM, NPARAM + NF
O_YMU, O_YSD = O_SD + NF, O_SD + NF + 1
NTOTAL = O_YSD + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[O_W1:O_B1].reshape(H, NF), p[O_B1:O_W2], p[O_W2:O_B2].reshape(H, H), p[O_B2:O_W3],
            p[O_W3:O_B3], p[O_B3], p[O_MU:O_SD], p[O_SD:O_YMU], p[O_YMU], p[O_YSD])


def forward(p, X):
    """log2(nnz) predictions for features X [n, 4]."""
    W1, b1, W2, b2, W3, b3, mu, sd, ymu, ysd = unpack(p)
    x = (np.asarray(X, np.float64) - mu) / sd
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return (h2 @ W3 + b3) * ysd + ymu


def loss_and_grad(p, X, y):
    """0.5 * sum (out - (y - ymu)/ysd)^2 and its gradient w.r.t. the first NPARAM entries."""
    W1, b1, W2, b2, W3, b3, mu, sd, ymu, ysd = unpack(p)
    x = (np.asarray(X, np.float64) - mu) / sd
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    o = h2 @ W3 + b3
    d = o - (np.asarray(y, np.float64) - ymu) / ysd
    loss = 0.5 * float(np.sum(d * d))
    dh2 = (z2 > 0) * (d[:, None] * W3[None, :])
    dh1 = (z1 > 0) * (dh2 @ W2)
    g = np.zeros(NPARAM)
    g[O_W1:O_B1] = (dh1.T @ x).reshape(-1)
    g[O_B1:O_W2] = dh1.sum(0)
    g[O_W2:O_B2] = (dh2.T @ h1).reshape(-1)
    g[O_B2:O_W3] = dh2.sum(0)
    g[O_W3:O_B3] = h2.T @ d
    g[O_B3] = d.sum()
    return loss, g
