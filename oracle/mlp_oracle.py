"""CPU oracle of the surrogate MLP (TEST INFRASTRUCTURE ONLY).

A numpy restatement of the network of include/spacelab_mlp.h: widths
padded to multiples of 32, BF16 rounding (round to nearest even) of the
GEMM operands -- weights, layer inputs, output gradients -- at the same
points as the GPU kernels, FP32 pre-activations, exact-erf GELU, MSE loss
over the real outputs.  Used by the tests to check the GPU forward pass and
gradients; it is never called by the library.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def pad32(x: int) -> int:
    return (x + 31) // 32 * 32


def layout(n_in: int, hidden: int, layers: int, n_out: int):
    din = [pad32(n_in)] + [pad32(hidden)] * layers
    dout = [pad32(hidden)] * layers + [pad32(n_out)]
    offs = []
    off = 0
    for a, b in zip(din, dout):
        offs.append((off, off + a * b))
        off += a * b + b
    return din, dout, offs, off


def unpack(params: np.ndarray, n_in, hidden, layers, n_out):
    din, dout, offs, _ = layout(n_in, hidden, layers, n_out)
    return [(params[w:w + a * b].reshape(b, a), params[bo:bo + b]) for (w, bo), a, b in zip(offs, din, dout)]


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(params, x, n_in, hidden, layers, n_out):
    Ws = unpack(params, n_in, hidden, layers, n_out)
    M = x.shape[0]
    X = np.zeros((M, Ws[0][0].shape[1]), dtype=np.float32)
    X[:, :n_in] = x
    X = bf16(X)
    Xs, Zs = [], []
    for l, (W, b) in enumerate(Ws):
        Xs.append(X)
        Z = (X.astype(np.float64) @ bf16(W).astype(np.float64).T + b).astype(np.float32)
        Zs.append(Z)
        if l < len(Ws) - 1:
            X = bf16(gelu(Z.astype(np.float64)).astype(np.float32))
    return Zs[-1][:, :n_out], Xs, Zs, Ws


def loss_and_grads(params, x, y, n_in, hidden, layers, n_out):
    out, Xs, Zs, Ws = forward(params, x, n_in, hidden, layers, n_out)
    M = x.shape[0]
    loss = float(((out.astype(np.float64) - y) ** 2).mean())
    dZ = np.zeros_like(Zs[-1])
    dZ[:, :n_out] = 2.0 * (Zs[-1][:, :n_out] - y) / (M * n_out)
    dZ = bf16(dZ)
    grads = np.zeros_like(params)
    din, dout, offs, _ = layout(n_in, hidden, layers, n_out)
    for l in range(len(Ws) - 1, -1, -1):
        (w0, b0), a, b = offs[l], din[l], dout[l]
        grads[w0:w0 + a * b] = (dZ.astype(np.float64).T @ Xs[l].astype(np.float64)).reshape(-1)
        grads[b0:b0 + b] = dZ.astype(np.float64).sum(0)
        if l == 0:
            break
        dX = dZ.astype(np.float64) @ bf16(Ws[l][0]).astype(np.float64)
        dZ = bf16((dX * gelu_grad(Zs[l - 1].astype(np.float64))).astype(np.float32))
    return loss, grads
