"""CPU oracle of the warm-start MLP (test infrastructure only).

An FP64 numpy restatement of the forward and backward passes that
``mlcp_gb300/mlp.py`` runs on the GPU, with the BF16 roundings at the same
points (inputs, weights as the GEMMs read them, hidden activations, the
loss gradient and the back-propagated pre-activation gradients), so that
the GPU's FP32-accumulated results can be compared with it.  With
``bf16=False`` it is the plain FP64 network, which the CPU tests check
against central finite differences.

The network: H1 = relu(X W1^T + b1), H2 = relu(H1 W2^T + b2),
Y = H2 W3^T + b3, loss = mean over the valid (rows x out) block of
(Y - T)^2.  There is no reference counterpart: the reference has no
learned component.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to BF16 (nearest, ties to even) and return as FP64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    out = ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)
    return out.astype(np.float64)


def forward(params, X, bf16_points: bool = True):
    """params = (W1, b1, W2, b2, W3, b3) in FP64 (logical shapes); X [rows][in].
    Returns (Y, cache)."""
    rd = bf16 if bf16_points else (lambda v: np.asarray(v, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = params
    Xr = rd(X)
    W1r, W2r, W3r = rd(W1), rd(W2), rd(W3)
    H1 = rd(np.maximum(Xr @ W1r.T + b1, 0.0))
    H2 = rd(np.maximum(H1 @ W2r.T + b2, 0.0))
    Y = H2 @ W3r.T + b3
    if bf16_points:
        Y = Y.astype(np.float32).astype(np.float64)
    return Y, (Xr, W1r, W2r, W3r, H1, H2)


def loss_and_grads(params, X, T, bf16_points: bool = True):
    """Mean squared error and its gradients (dW1, db1, dW2, db2, dW3, db3)."""
    rd = bf16 if bf16_points else (lambda v: np.asarray(v, dtype=np.float64))
    Y, (Xr, W1r, W2r, W3r, H1, H2) = forward(params, X, bf16_points)
    m, n = Y.shape
    diff = Y - T
    loss = float(np.mean(diff ** 2))
    dY = rd(2.0 * diff / (m * n))
    dW3 = dY.T @ H2
    db3 = dY.sum(axis=0)
    dZ2 = rd((dY @ W3r) * (H2 > 0))
    dW2 = dZ2.T @ H1
    db2 = dZ2.sum(axis=0)
    dZ1 = rd((dZ2 @ W2r) * (H1 > 0))
    dW1 = dZ1.T @ Xr
    db1 = dZ1.sum(axis=0)
    return loss, [dW1, db1, dW2, db2, dW3, db3]


def finite_difference(params, X, T, which: int, index, h: float = 1e-6) -> float:
    """Central difference of the FP64 loss with respect to params[which][index]."""
    p_plus = [p.copy() for p in params]
    p_minus = [p.copy() for p in params]
    p_plus[which][index] += h
    p_minus[which][index] -= h
    lp, _ = loss_and_grads(p_plus, X, T, bf16_points=False)
    lm, _ = loss_and_grads(p_minus, X, T, bf16_points=False)
    return (lp - lm) / (2 * h)
