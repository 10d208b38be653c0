"""CPU restatement (numpy, FP64) of the warm-start network of
superdca_gb300/csrc/mlp.cu -- test infrastructure only, used to check the
GPU forward and backward kernels.

SuperDCA has no learned component, so this restates this project's own
network: input normalisation (x - mean) * scale, two ReLU layers of 128 and
a linear layer of 16; loss = mean over rows of the summed squared error.
The blob layout is the one documented in include/superdca_gb300.h."""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT = 40, 128, 16
IN_MEAN, IN_SCALE = 4, 4 + N_IN
W1 = IN_SCALE + N_IN
B1 = W1 + N_H * N_IN
W2 = B1 + N_H
B2 = W2 + N_H * N_H
W3 = B2 + N_H
B3 = W3 + N_OUT * N_H
TRAIN_END = B3 + N_OUT
SIZE = TRAIN_END + N_OUT


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(mean=p[IN_MEAN:IN_MEAN + N_IN], scale=p[IN_SCALE:IN_SCALE + N_IN],
                W1=p[W1:B1].reshape(N_H, N_IN), b1=p[B1:W2], W2=p[W2:B2].reshape(N_H, N_H), b2=p[B2:W3],
                W3=p[W3:B3].reshape(N_OUT, N_H), b3=p[B3:TRAIN_END])


def forward(p, X):
    q = unpack(p)
    xn = (np.asarray(X, dtype=np.float64) - q["mean"]) * q["scale"]
    h1 = np.maximum(xn @ q["W1"].T + q["b1"], 0.0)
    h2 = np.maximum(h1 @ q["W2"].T + q["b2"], 0.0)
    return xn, h1, h2, h2 @ q["W3"].T + q["b3"]


def loss_and_grad(p, X, T):
    q = unpack(p)
    xn, h1, h2, out = forward(p, X)
    M = len(X)
    r = out - np.asarray(T, dtype=np.float64)
    loss = (r * r).sum() / M
    d3 = 2.0 * r / M
    g = np.zeros(SIZE)
    g[W3:B3] = (d3.T @ h2).ravel()
    g[B3:TRAIN_END] = d3.sum(0)
    d2 = (d3 @ q["W3"]) * (h2 > 0)
    g[W2:B2] = (d2.T @ h1).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = (d2 @ q["W2"]) * (h1 > 0)
    g[W1:B1] = (d1.T @ xn).ravel()
    g[B1:W2] = d1.sum(0)
    return loss, g


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def forward_bf16(p, X):
    """The tensor-core forward's arithmetic: normalised inputs, weights and
    hidden activations rounded to bfloat16, sums and biases in full
    precision (the kernel accumulates in FP32)."""
    q = unpack(np.asarray(p, dtype=np.float32))
    xn = (np.asarray(X, dtype=np.float32) - q["mean"].astype(np.float32)) * q["scale"].astype(np.float32)
    a1 = bf16(xn).astype(np.float64)
    h1 = np.maximum(a1 @ bf16(q["W1"]).astype(np.float64).T + q["b1"], 0.0)
    a2 = bf16(h1).astype(np.float64)
    h2 = np.maximum(a2 @ bf16(q["W2"]).astype(np.float64).T + q["b2"], 0.0)
    a3 = bf16(h2).astype(np.float64)
    return a3 @ bf16(q["W3"]).astype(np.float64).T + q["b3"]
