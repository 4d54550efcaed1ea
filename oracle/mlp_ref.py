"""CPU restatement of the integrand-surrogate network, for checking the GPU
kernels' forward pass and gradients. TEST INFRASTRUCTURE ONLY (see
oracle/ac_cas_ref.py).

Same conventions as the library: layers in -> H -> H -> H -> out, exact-erf
GELU on hidden layers, forward and data gradient through BF16-rounded weights
(round to nearest even), biases FP32, MSE loss mean over batch x out, weight
gradients taken as if the weights were their BF16 values. Arithmetic in FP64.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16_round(x: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unflatten(p: np.ndarray, dims):
    out, off = [], 0
    for l in range(len(dims) - 1):
        din, dout = dims[l], dims[l + 1]
        W = p[off:off + din * dout].reshape(dout, din)
        off += din * dout
        b = p[off:off + dout]
        off += dout
        out.append((W, b))
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def forward(p, dims, x):
    layers = unflatten(np.asarray(p, dtype=np.float64), dims)
    h = np.asarray(x, dtype=np.float64)
    zs, hs = [], [h]
    for l, (W, b) in enumerate(layers):
        z = h @ bf16_round(W).T + b
        zs.append(z)
        h = z if l == len(layers) - 1 else gelu(z)
        hs.append(h)
    return h, zs, hs


def loss_and_grad(p, dims, x, t):
    y, zs, hs = forward(p, dims, x)
    layers = unflatten(np.asarray(p, dtype=np.float64), dims)
    n = y.size
    loss = np.sum((y - t) ** 2) / n
    dz = 2.0 * (y - t) / n
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        grads.append((dz.T @ hs[l], dz.sum(axis=0)))
        if l == 0:
            break
        dh = dz @ bf16_round(W)
        dz = dh * gelu_grad(zs[l - 1])
    grads = grads[::-1]
    return loss, np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
