"""CPU restatement of the learned Newton start value's network -- TEST
INFRASTRUCTURE ONLY (imported by tests/, never by the product path).

The reference has no counterpart: its ExactRiemannSolver starts Newton's
iteration from the mean pressure (src/equations/perfect_gas/
ExactRiemannSolver.hpp:34-97).  This module states the 5 -> 64 -> 64 -> 1
GELU perceptron, its mean-squared-error loss and its gradients in float64
numpy, so that the device's forward pass, backward pass and Adam step can be
checked against it.  With ``bf16_operands=True`` the operands are rounded to bfloat16
at the points where the device feeds the tensor cores (standardised inputs,
W1, W2, the first hidden activation, and the two back-propagated signals);
everything else stays float64.  Parity of this restatement is pinned by
finite differences of its own loss (the analytic gradient matches central
differences in float64), not by a reference implementation.

Parameter blob layout (floats): mean[5], inv_std[5], W1[64][5], b1[64],
W2[64][64], b2[64], w3[64], b3.
"""
from __future__ import annotations

import numpy as np

N_IN = 5
HIDDEN = 64
OFF_MEAN = 0
OFF_INVSTD = OFF_MEAN + N_IN
OFF_W1 = OFF_INVSTD + N_IN
OFF_B1 = OFF_W1 + HIDDEN * N_IN
OFF_W2 = OFF_B1 + HIDDEN
OFF_B2 = OFF_W2 + HIDDEN * HIDDEN
OFF_W3 = OFF_B2 + HIDDEN
OFF_B3 = OFF_W3 + HIDDEN
N_PARAMS = OFF_B3 + 1

_K0 = 0.7978845608028654
_K1 = 0.044715


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as
    float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_K0 * (x + _K1 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(_K0 * (x + _K1 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _K0 * (1.0 + 3.0 * _K1 * x * x)


def features(gamma, rhoL, uL, pL, rhoR, uR, pR):
    """x0 = log(rhoR/rhoL), x1 = log(pR/pL), x2 = (uR-uL)/c, x3 = aL/c,
    x4 = aR/c with c = max(aL, aR); float32 [n, 5]."""
    aL = np.sqrt(gamma * pL / rhoL)
    aR = np.sqrt(gamma * pR / rhoR)
    c = np.maximum(aL, aR)
    f = np.stack([np.log(rhoR / rhoL), np.log(pR / pL), (uR - uL) / c, aL / c, aR / c], axis=1)
    return f.astype(np.float32)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(
        mean=p[OFF_MEAN:OFF_MEAN + N_IN], inv_std=p[OFF_INVSTD:OFF_INVSTD + N_IN],
        W1=p[OFF_W1:OFF_B1].reshape(HIDDEN, N_IN), b1=p[OFF_B1:OFF_W2],
        W2=p[OFF_W2:OFF_B2].reshape(HIDDEN, HIDDEN), b2=p[OFF_B2:OFF_W3],
        w3=p[OFF_W3:OFF_B3], b3=p[OFF_B3])


def forward(p, feat, bf16_operands=False):
    """Network output y [n] for raw features [n, 5]."""
    y, _ = _forward(p, feat, bf16_operands)
    return y


def _forward(p, feat, rb):
    w = unpack(p)
    r = bf16 if rb else (lambda v: np.asarray(v, dtype=np.float64))
    x = (np.asarray(feat, np.float32) - w["mean"].astype(np.float32)) * w["inv_std"].astype(np.float32)
    X = r(x)
    W1 = bf16(w["W1"].astype(np.float32)) if rb else w["W1"]
    W2 = bf16(w["W2"].astype(np.float32)) if rb else w["W2"]
    Z1 = X @ W1.T + w["b1"]
    H1 = r(gelu(Z1).astype(np.float32)) if rb else gelu(Z1)
    Z2 = H1 @ W2.T + w["b2"]
    H2 = gelu(Z2)
    y = H2 @ w["w3"] + w["b3"]
    return y, dict(X=X, W1=W1, W2=W2, Z1=Z1, H1=H1, Z2=Z2, H2=H2, w=w)


def loss_and_grad(p, feat, label, bf16_operands=False):
    """Mean squared error over the rows and its gradient in the blob layout
    (the normalisation entries get 0)."""
    rb = bf16_operands
    y, c = _forward(p, feat, rb)
    n = len(y)
    e = y - np.asarray(label, dtype=np.float64)
    loss = float(np.mean(e * e))
    dy = 2.0 * e / n
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = c["H2"].T @ dy
    g[OFF_B3] = dy.sum()
    d2 = dy[:, None] * c["w"]["w3"][None, :] * gelu_grad(c["Z2"])
    g[OFF_B2:OFF_W3] = d2.sum(axis=0)
    D2 = bf16(d2.astype(np.float32)) if rb else d2
    g[OFF_W2:OFF_B2] = (D2.T @ c["H1"]).ravel()
    dH1 = D2 @ c["W2"]
    d1 = dH1 * gelu_grad(c["Z1"])
    g[OFF_B1:OFF_W2] = d1.sum(axis=0)
    D1 = bf16(d1.astype(np.float32)) if rb else d1
    g[OFF_W1:OFF_B1] = (D1.T @ c["X"]).ravel()
    return loss, g


def adam_step(p, g, m1, m2, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (t counts from 1) on the weights and biases; the
    normalisation entries are left alone.  Returns new (p, m1, m2)."""
    p = np.array(p, dtype=np.float64)
    m1 = beta1 * m1 + (1 - beta1) * g
    m2 = beta2 * m2 + (1 - beta2) * g * g
    mh = m1 / (1 - beta1 ** t)
    vh = m2 / (1 - beta2 ** t)
    upd = lr * mh / (np.sqrt(vh) + eps)
    upd[:OFF_W1] = 0.0
    return p - upd, m1, m2
