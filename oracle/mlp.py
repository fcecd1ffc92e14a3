"""Numpy forward/backward of the learned-start MLP -- TEST INFRASTRUCTURE
ONLY: the gradient oracle for tupan_gb300/csrc/mlp.cu.

Network: x (4 features, normalised with mean/1-over-std) -> 64 SiLU -> 64
SiLU -> 1, loss = scale * sum (y - target)^2 over samples with a finite
target.  Parameters use the flat layout of mlp.cu: W1 (64x4), b1, W2
(64x64), b2, w3 (64), b3.
"""

import numpy as np

IN, H = 4, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
N_PARAM = OFF_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, IN), p[OFF_B1:OFF_W2],
            p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def sig(x):
    return 1.0 / (1.0 + np.exp(-x))


def forward(p, norm, X):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = (np.asarray(X, np.float64) - norm[:4]) * norm[4:]
    z1 = x @ W1.T + b1
    h1 = z1 * sig(z1)
    z2 = h1 @ W2.T + b2
    h2 = z2 * sig(z2)
    return h2 @ w3 + b3, (x, z1, h1, z2, h2)


def grad(p, norm, X, Y, scale):
    """Gradient of scale * sum (y - t)^2 and the sum of squared errors."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    y, (x, z1, h1, z2, h2) = forward(p, norm, X)
    Y = np.asarray(Y, np.float64)
    ok = np.isfinite(Y)
    err = np.where(ok, y - np.where(ok, Y, 0.0), 0.0)
    g = 2.0 * err * scale
    x = np.where(ok[:, None], x, 0.0)
    dsilu = lambda z: sig(z) * (1.0 + z * (1.0 - sig(z)))
    d2 = g[:, None] * w3[None, :] * dsilu(z2)
    d1 = (d2 @ W2) * dsilu(z1)
    out = np.zeros(N_PARAM)
    out[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    out[OFF_B1:OFF_W2] = d1.sum(0)
    out[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    out[OFF_B2:OFF_W3] = d2.sum(0)
    out[OFF_W3:OFF_B3] = h2.T @ g
    out[OFF_B3] = g.sum()
    return out, float((err ** 2).sum())
