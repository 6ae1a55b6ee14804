"""TEST INFRASTRUCTURE -- the CPU oracle of the order controller's network,
never the product.

A numpy FP64 restatement of the 16-64-64-5 ReLU MLP the library trains and
evaluates on the GPU (csrc/mlp.cu, csrc/ctrl_mma.cuh): forward pass with the
kernels' BF16 rounding of weights (and, optionally, of the normalised inputs
and hidden activations, as the tensor-core inference does), and the
mean-squared-error loss with its analytic gradient.  The gradient is pinned
by central finite differences (tests/test_mlp_reference.py); the GPU training
and inference kernels are checked against it (tests/test_gpu_learned.py).
The parameter layout is the library's: W1 (64x16), b1, W2 (64x64), b2,
W3 (5x64), b3, concatenated.
"""
from __future__ import annotations

import numpy as np

NPARAM = 64 * 16 + 64 + 64 * 64 + 64 + 5 * 64 + 5


def bf16(x):
    """Round-to-nearest-even to bfloat16, kept in float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    o = 0
    W1 = p[o:o + 1024].reshape(64, 16); o += 1024
    b1 = p[o:o + 64]; o += 64
    W2 = p[o:o + 4096].reshape(64, 64); o += 4096
    b2 = p[o:o + 64]; o += 64
    W3 = p[o:o + 320].reshape(5, 64); o += 320
    b3 = p[o:o + 5]
    return W1, b1, W2, b2, W3, b3


def reference_forward(p, X, mean, std, round_activations=False):
    """Forward pass with BF16-rounded weights (FP64 arithmetic); with
    round_activations the normalised inputs and the hidden activations are
    rounded to BF16 too, as the list builder's tensor-core evaluation does."""
    r = bf16 if round_activations else (lambda a: a)
    W1, b1, W2, b2, W3, b3 = [a.astype(np.float64) for a in unpack(bf16(p))]
    x = r(((X - mean) * (1.0 / std).astype(np.float32)).astype(np.float32)).astype(np.float64)
    h1 = r(np.maximum(x @ W1.T + b1, 0).astype(np.float32)).astype(np.float64)
    h2 = r(np.maximum(h1 @ W2.T + b2, 0).astype(np.float32)).astype(np.float64)
    return h2 @ W3.T + b3


def reference_loss_grad(p, X, T, mean, std, round_weights=True, dtype=np.float64):
    """Mean-squared-error loss and its gradient w.r.t. the (rounded) parameters."""
    q = bf16(p) if round_weights else p
    W1, b1, W2, b2, W3, b3 = [a.astype(dtype) for a in unpack(q.astype(dtype))]
    x = ((X - mean) / std).astype(dtype)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    y = h2 @ W3.T + b3
    e = y - T
    n = e.size
    loss = float((e ** 2).sum() / n)
    dy = 2 * e / n
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    d2 = (dy @ W3) * (z2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (z1 > 0)
    gW1 = d1.T @ x
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
