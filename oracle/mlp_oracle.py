"""CPU oracle for the surrogate MLP's forward and backward pass.

TEST INFRASTRUCTURE ONLY (the checker of the GPU kernels; never on the product path).

Float64 NumPy restatement of the network the rbf_mlp_* kernels run: y = W_L g(... g(W_1 x + b_1)
...) + b_L with the GELU g in its tanh form, MSE loss mean((y - t)^2) over the real output columns,
and its gradients by reverse-mode differentiation.  The GPU keeps matrices, activations and
back-propagated signals in bf16; the same roundings are applied here at the same places
(`bf16` below), so the two differ only by FP32-vs-FP64 accumulation.
"""
import math

import numpy as np


def bf16(a):
    """Round float32 values to bf16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    """GELU in its tanh form (Hendrycks & Gimpel), the activation of the surrogate."""
    u = math.sqrt(2.0 / math.pi) * (z + 0.044715 * z ** 3)
    return 0.5 * z * (1.0 + np.tanh(u))


def gelu_grad(z):
    c = math.sqrt(2.0 / math.pi)
    t = np.tanh(c * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * c * (1.0 + 3 * 0.044715 * z * z)


def forward_backward(X, W, b, T, dout):
    """X: bf16-valued inputs (B x din_pad), W/b: lists of FP32 parameters, T: targets (B x dout_pad).
    Returns loss, y, [dW], [db] in float64."""
    L = len(W)
    Wb = [bf16(w) for w in W]
    acts, zs = [np.asarray(X, dtype=np.float64)], []
    a = acts[0]
    for i in range(L):
        z = a @ Wb[i].T + b[i]
        if i < L - 1:
            zs.append(z)
            a = bf16(gelu(z))
            acts.append(a)
        else:
            y = z
    B = X.shape[0]
    sc = 1.0 / (B * dout)
    d = np.zeros_like(y)
    d[:, :dout] = y[:, :dout] - T[:, :dout]
    loss = float((d ** 2).sum() * sc)
    dz = bf16(2.0 * d * sc)
    dW, db = [None] * L, [None] * L
    for i in range(L - 1, -1, -1):
        dW[i] = dz.T @ acts[i]
        db[i] = dz.sum(axis=0)
        if i > 0:
            dz = bf16((dz @ Wb[i]) * gelu_grad(zs[i - 1]))
    return loss, y, dW, db
