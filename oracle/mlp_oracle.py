"""FP64 NumPy restatement of the early-exit network's objective and gradient.

TEST INFRASTRUCTURE ONLY: the CPU restatement that the hand-written CUDA training
kernels (song_gb300/csrc/mlp.cu) are compared with.  Network 5 -> 32 -> 32 -> 1 with ReLU
(derivative 0 at 0), loss = sum_i w_i (softplus(z_i) - y_i z_i) / sum_i w_i,
parameters in the SONG_MLP_PARAMS layout W1[32][5], b1[32], W2[32][32],
b2[32], w3[32], b3.
"""
import numpy as np

NPARAM = 1281


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[0:160].reshape(32, 5), p[160:192], p[192:1216].reshape(32, 32), p[1216:1248],
            p[1248:1280], p[1280])


def forward(x, p):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ w3 + b3
    return z, (x, a1, h1, a2, h2)


def loss_and_grad(x, y, p, w=None):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    z, (x, a1, h1, a2, h2) = forward(x, p)
    y = np.asarray(y, dtype=np.float64)
    w = np.ones_like(y) if w is None else np.asarray(w, dtype=np.float64)
    wt = w.sum()
    sp = np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))
    loss = float((w * (sp - y * z)).sum() / wt)
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y) / wt
    g_b3 = dz.sum()
    g_w3 = h2.T @ dz
    da2 = (dz[:, None] * w3[None, :]) * (a2 > 0)
    g_b2 = da2.sum(0)
    g_W2 = da2.T @ h1
    dh1 = da2 @ W2
    da1 = dh1 * (a1 > 0)
    g_b1 = da1.sum(0)
    g_W1 = da1.T @ x
    g = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, g
