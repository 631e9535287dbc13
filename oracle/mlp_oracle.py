"""
CPU checker for the learned-depth part (TEST INFRASTRUCTURE ONLY; only tests/
may import it).

- mlp_forward / mlp_grad: NumPy float64 forward pass and mean-squared-loss
  gradient of the 12 -> 64 -> 64 -> 1 GELU network, same parameter layout as the
  device kernels (W1[64][12], b1[64], W2[64][64], b2[64], W3[64], b3).
- depth_label: the label rule (smallest Krylov depth m whose a-posteriori
  estimate beta_m |e_m^T exp(dt T_m) e_1| is below tol) from a record's alpha /
  beta, with numpy.linalg.eigh for the tridiagonal matrices, as
  pytenet/krylov.py:122-150 forms exp(dt T) e_1.
"""

import numpy as np
from math import erf, sqrt, pi

_erf = np.vectorize(erf)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    w1 = p[o:o + 768].reshape(64, 12); o += 768
    b1 = p[o:o + 64]; o += 64
    w2 = p[o:o + 4096].reshape(64, 64); o += 4096
    b2 = p[o:o + 64]; o += 64
    w3 = p[o:o + 64]; o += 64
    b3 = p[o]
    return w1, b1, w2, b2, w3, b3


def gelu(x):
    return 0.5 * x * (1 + _erf(x / sqrt(2)))


def gelu_grad(x):
    return 0.5 * (1 + _erf(x / sqrt(2))) + x * np.exp(-0.5 * x * x) / sqrt(2 * pi)


def mlp_forward(p, X):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    z1 = X @ w1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ w2.T + b2
    h2 = gelu(z2)
    return h2 @ w3 + b3


def mlp_grad(p, X, T):
    """Gradient of mean((y - T)^2) with respect to the flat parameter vector."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[0]
    z1 = X @ w1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ w2.T + b2
    h2 = gelu(z2)
    y = h2 @ w3 + b3
    dy = 2 * (y - T) / B
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = np.outer(dy, w3) * gelu_grad(z2)
    gw2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ w2) * gelu_grad(z1)
    gw1 = dz1.T @ X
    gb1 = dz1.sum(0)
    loss = np.mean((y - T) ** 2)
    return np.concatenate([gw1.ravel(), gb1, gw2.ravel(), gb2, gw3, [gb3]]), loss


def depth_label(rec, m_max=20, tol=1e-10):
    """Label of one training record laid out as written by the device
    (features[12], alpha[24], beta[24] with beta[m_used-1] the final residual
    norm, nrm, dt_re, dt_im, m_used)."""
    alpha = rec[12:36]
    beta = rec[36:60]
    nrm, dt = rec[60], complex(rec[61], rec[62])
    mu = min(int(rec[63]), m_max, 24)
    for m in range(1, mu + 1):
        t = np.diag(alpha[:m]) + np.diag(beta[:m - 1], 1) + np.diag(beta[:m - 1], -1)
        w, u = np.linalg.eigh(t)
        c = u @ (nrm * np.exp(dt * w) * u[0])
        if beta[m - 1] * abs(c[m - 1]) / nrm <= tol:
            return m
    return m_max
