"""CPU oracle of the learned block-Jacobi correction -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy FP64, the per-node MLP (16 -> 64 -> 64 -> 6, SiLU) with the same BF16
rounding points as the GPU path (weights, inputs and hidden activations rounded to BF16;
pre-activations accumulated exactly), the probe loss and its gradient, and the
preconditioner blocks P_i = G_i^{-T} L L^T G_i^{-1}.  The MLP has no reference counterpart;
this is the checker for the hand-written forward (tensor cores) and backward kernels.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT, N_USED = 16, 64, 16, 6


def bf16_round(x):
    """Round-to-nearest-even FP32 -> BF16 -> FP32 (as __float2bfloat16_rn)."""
    a = np.asarray(x, dtype=np.float32).copy()
    b = a.view(np.uint32)
    lsb = (b >> 16) & 1
    b = (b + 0x7FFF + lsb) & 0xFFFF0000
    return b.view(np.float32).astype(np.float64)


def bf16_bits(x):
    a = np.asarray(x, dtype=np.float32).copy()
    b = a.view(np.uint32)
    lsb = (b >> 16) & 1
    return (((b + 0x7FFF + lsb) >> 16) & 0xFFFF).astype(np.uint16)


def bits_to_float(u16):
    return (np.asarray(u16, dtype=np.uint32) << 16).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_HID * N_IN].reshape(N_HID, N_IN); o += N_HID * N_IN
    b1 = p[o:o + N_HID]; o += N_HID
    W2 = p[o:o + N_HID * N_HID].reshape(N_HID, N_HID); o += N_HID * N_HID
    b2 = p[o:o + N_HID]; o += N_HID
    W3 = p[o:o + N_OUT * N_HID].reshape(N_OUT, N_HID); o += N_OUT * N_HID
    b3 = p[o:o + N_OUT]
    return W1, b1, W2, b2, W3, b3


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, X):
    """X: (n,16) FP32 values already representable in BF16.  Returns out, z1, z2, h1, h2."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W1, W2, W3 = bf16_round(W1), bf16_round(W2), bf16_round(W3)
    z1 = X @ W1.T + b1
    h1 = bf16_round(silu(z1))
    z2 = h1 @ W2.T + b2
    h2 = bf16_round(silu(z2))
    out = h2 @ W3.T + b3
    return out, z1, z2, h1, h2


def lower(o):
    L = np.zeros(o.shape[:-1] + (3, 3))
    L[..., 0, 0] = np.exp(o[..., 0])
    L[..., 1, 1] = np.exp(o[..., 1])
    L[..., 2, 2] = np.exp(o[..., 2])
    L[..., 1, 0] = o[..., 3]
    L[..., 2, 0] = o[..., 4]
    L[..., 2, 1] = o[..., 5]
    return L


def loss_grad(out, yhat, zhat):
    """out (n,16); yhat, zhat (n,3,R).  loss = mean_{i,r} |C y - z|^2; returns (loss, dout)."""
    n, _, R = yhat.shape
    L = lower(out)
    C = L @ np.swapaxes(L, 1, 2)
    e = C @ yhat - zhat                                     # (n,3,R)
    loss = np.sum(e * e) / (n * R)
    G = 2.0 * e @ np.swapaxes(yhat, 1, 2) / (n * R)         # dloss/dC
    dL = (G + np.swapaxes(G, 1, 2)) @ L
    d = np.zeros_like(out)
    d[:, 0] = dL[:, 0, 0] * L[:, 0, 0]
    d[:, 1] = dL[:, 1, 1] * L[:, 1, 1]
    d[:, 2] = dL[:, 2, 2] * L[:, 2, 2]
    d[:, 3] = dL[:, 1, 0]
    d[:, 4] = dL[:, 2, 0]
    d[:, 5] = dL[:, 2, 1]
    return loss, d


def backward(params, X, z1, z2, dout):
    """Parameter gradient (flat, same order as the FP32 parameter vector)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W2r, W3r = bf16_round(W2), bf16_round(W3)
    h1 = bf16_round(silu(z1))
    h2 = bf16_round(silu(z2))
    d3 = np.zeros_like(dout)
    d3[:, :N_USED] = dout[:, :N_USED]
    dz2 = (d3[:, :N_USED] @ W3r[:N_USED]) * silu_grad(z2)
    dz1 = (dz2 @ W2r) * silu_grad(z1)
    gW3 = np.zeros((N_OUT, N_HID))
    gW3[:N_USED] = d3[:, :N_USED].T @ h2
    gb3 = np.zeros(N_OUT)
    gb3[:N_USED] = d3[:, :N_USED].sum(0)
    return np.concatenate([(dz1.T @ X).ravel(), dz1.sum(0), (dz2.T @ h1).ravel(), dz2.sum(0), gW3.ravel(), gb3])


def backward_bf16(params, X, z1, z2, dout):
    """The parameter gradient with the rounding points of the tensor-core backward
    (fem_mlp_backward_tc): dz3, dz2 = (dz3 W3) s2' and dz1 = (bf16(dz2) W2) s1' are rounded to
    BF16 where they become matrix-product operands; sums are exact here (FP32 on the GPU)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W2r, W3r = bf16_round(W2), bf16_round(W3)
    h1 = bf16_round(silu(z1))
    h2 = bf16_round(silu(z2))
    d3 = np.asarray(dout, dtype=np.float64)[:, :N_USED]
    dz2 = bf16_round((d3 @ W3r[:N_USED]) * silu_grad(z2))
    dz1 = bf16_round((dz2 @ W2r) * silu_grad(z1))
    d3b = bf16_round(d3)
    gW3 = np.zeros((N_OUT, N_HID))
    gW3[:N_USED] = d3b.T @ h2
    gb3 = np.zeros(N_OUT)
    gb3[:N_USED] = d3b.sum(0)
    return np.concatenate([(dz1.T @ X).ravel(), dz1.sum(0), (dz2.T @ h1).ravel(), dz2.sum(0), gW3.ravel(), gb3])


def precond_blocks(out, ginv):
    """P = G^{-T} C G^{-1} with C = L L^T; ginv (n,3,3) lower-triangular."""
    L = lower(out)
    C = L @ np.swapaxes(L, 1, 2)
    return np.swapaxes(ginv, 1, 2) @ C @ ginv
