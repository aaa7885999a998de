"""CPU restatement (float64 accumulation, BF16 rounding where the device rounds) of the
learned-closure MLP of fsi/closure.py, used only by the tests as the checker of the
tensor-core GEMMs, the fused inference and the gradients.

Network: 656 -> 64 -> 64 -> 64 -> 32 (19 used), GELU (tanh form of Hendrycks & Gimpel
2016), BF16 weights and activations, FP32/float64 accumulation. There is no reference
counterpart to pin it to: the device path is checked against this restatement.
"""
from __future__ import annotations

import numpy as np

C0 = 0.7978845608028654
C1 = 0.044715


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even) and back to float64."""
    a = np.asarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(C0 * (z + C1 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(C0 * (z + C1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * C0 * (1.0 + 3.0 * C1 * z * z)


def forward(x, W1, b1, W2, b2, W3, b3, W4):
    """x: [m, 656] (already BF16 values); returns y [m, 32] and the activations."""
    acts = []
    h = np.asarray(x, np.float64)
    for W, b in ((W1, b1), (W2, b2), (W3, b3)):
        z = h @ bf16(W).T + np.asarray(b, np.float64)
        z32 = z.astype(np.float32).astype(np.float64)
        h = bf16(gelu(z32))
        acts.append((z32, h))
    y = h @ bf16(W4).T
    return y, acts


def backward(x, y, acts, target, W2, W3, W4, b4):
    """Gradients of mean((y[:, :19] + b4[:19] - target)^2) as the device computes them."""
    m = x.shape[0]
    e = y[:, :19] + np.asarray(b4, np.float64)[:19] - target
    loss = float(np.mean(e ** 2))
    dy = np.zeros((m, 32))
    dy[:, :19] = bf16(2.0 * e / (m * 19))
    grads = {"W4": dy.T @ acts[2][1], "b4": dy.sum(0)}
    g = dy
    for layer, Wup in ((3, W4), (2, W3), (1, W2)):
        z, _ = acts[layer - 1]
        dz = bf16((g @ bf16(Wup)) * gelu_grad(z))
        below = x if layer == 1 else acts[layer - 2][1]
        grads[f"W{layer}"] = dz.T @ below
        grads[f"b{layer}"] = dz.sum(0)
        g = dz
    return loss, grads
