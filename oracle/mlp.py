"""Oracle (test infrastructure only) for the learned EM warm start network.

CPU restatement, in float64 numpy, of the network that pcaone_gb300/csrc/mlp.cu
trains on the GPU: x[64] -> 256 (ReLU) -> 256 (ReLU) -> 1, mean squared error.
The GPU forward pass uses the BF16 rounding of the weights (round to nearest,
ties to even); `bf16` reproduces that rounding so the outputs and the
gradients (taken with respect to the rounded weights) can be compared
directly.  The warm start has no counterpart in the reference; its EM loop is
src/Halko.cpp:290-320, whose mean-fill start the network replaces.

Parameter layout (float32, 82,689 values): W1 [64 x 256] (row = input), b1 [256],
W2 [256 x 256], b2 [256], w3 [256], b3 [1].
"""
from __future__ import annotations

import numpy as np

N_IN, N_H = 64, 256
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_IN * N_H
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_H
N_PARAMS = OFF_B3 + 1


def bf16(a: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def unpack(theta: np.ndarray, round_weights: bool = True):
    t = np.asarray(theta, dtype=np.float32)
    rw = bf16 if round_weights else (lambda v: v)
    W1 = rw(t[OFF_W1:OFF_B1]).reshape(N_IN, N_H).astype(np.float64)
    b1 = t[OFF_B1:OFF_W2].astype(np.float64)
    W2 = rw(t[OFF_W2:OFF_B2]).reshape(N_H, N_H).astype(np.float64)
    b2 = t[OFF_B2:OFF_W3].astype(np.float64)
    w3 = rw(t[OFF_W3:OFF_B3]).astype(np.float64)
    b3 = float(t[OFF_B3])
    return W1, b1, W2, b2, w3, b3


def forward_backward(X: np.ndarray, y: np.ndarray, theta: np.ndarray, round_weights: bool = True):
    """Returns (out, loss, grads) like pcaone_gpu_mlp_forward_backward."""
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    B = X.shape[0]
    W1, b1, W2, b2, w3, b3 = unpack(theta, round_weights)
    A1 = np.maximum(X @ W1 + b1, 0.0)
    A2 = np.maximum(A1 @ W2 + b2, 0.0)
    out = A2 @ w3 + b3
    e = out - y
    loss = float(np.mean(e * e))
    dout = 2.0 * e / B
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = A2.T @ dout
    g[OFF_B3] = dout.sum()
    dZ2 = np.outer(dout, w3) * (A2 > 0)
    g[OFF_W2:OFF_B2] = (A1.T @ dZ2).ravel()
    g[OFF_B2:OFF_W3] = dZ2.sum(0)
    dZ1 = (dZ2 @ W2.T) * (A1 > 0)
    g[OFF_W1:OFF_B1] = (X.T @ dZ1).ravel()
    g[OFF_B1:OFF_W2] = dZ1.sum(0)
    return out, loss, g


def he_init(seed: int) -> np.ndarray:
    """He-uniform weights and zero biases (a test initialisation)."""
    rng = np.random.default_rng(seed)
    t = np.zeros(N_PARAMS, dtype=np.float32)
    t[OFF_W1:OFF_B1] = rng.uniform(-1, 1, N_IN * N_H) * np.sqrt(6.0 / N_IN)
    t[OFF_W2:OFF_B2] = rng.uniform(-1, 1, N_H * N_H) * np.sqrt(6.0 / N_H)
    t[OFF_W3:OFF_B3] = rng.uniform(-1, 1, N_H) * np.sqrt(3.0 / N_H)
    t[OFF_B1:OFF_W2] = rng.uniform(-0.1, 0.1, N_H)
    t[OFF_B2:OFF_W3] = rng.uniform(-0.1, 0.1, N_H)
    t[OFF_B3] = 0.05
    return t
