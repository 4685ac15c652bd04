"""numpy restatement of the surrogate MLP (test infrastructure): forward and
backward propagation of nin -> nh -> nh -> nout with SiLU and the mean
squared error of standardised outputs, in float64, for checking the GPU
gradient kernels.  Parameter vector layout: [W1 (nh x nin), b1, W2 (nh x nh),
b2, W3 (nout x nh), b3]."""
from __future__ import annotations

import numpy as np


def unpack(P, nin, nh, nout):
    P = np.asarray(P, dtype=np.float64)
    o = 0
    out = []
    for r, c in ((nh, nin), (nh, nh), (nout, nh)):
        out.append(P[o:o + r * c].reshape(r, c))
        o += r * c
        out.append(P[o:o + r])
        o += r
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(P, X, nin, nh, nout):
    W1, b1, W2, b2, W3, b3 = unpack(P, nin, nh, nout)
    X = np.asarray(X, dtype=np.float64)
    Z1 = X @ W1.T + b1
    H1 = silu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = silu(Z2)
    return H2 @ W3.T + b3, (X, Z1, H1, Z2, H2)


def gradients(P, X, Yt, shift, scale, nin, nh, nout):
    """Gradient of mean((Y - (Yt - shift)/scale)^2) with respect to P."""
    W1, b1, W2, b2, W3, b3 = unpack(P, nin, nh, nout)
    Y, (X, Z1, H1, Z2, H2) = forward(P, X, nin, nh, nout)
    T = (np.asarray(Yt, dtype=np.float64) - shift) / scale
    R = Y - T
    dY = 2.0 * R / R.size
    gW3 = dY.T @ H2
    gb3 = dY.sum(0)
    dZ2 = (dY @ W3) * silu_grad(Z2)
    gW2 = dZ2.T @ H1
    gb2 = dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * silu_grad(Z1)
    gW1 = dZ1.T @ X
    gb1 = dZ1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return g, float(np.mean(R * R))
