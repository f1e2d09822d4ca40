"""NumPy restatement of the learned smoother's network for the gradient
check (TEST INFRASTRUCTURE ONLY).

Same parameter layout and arithmetic as the GPU kernels: operands of every
GEMM rounded to BF16 (round to nearest even), FP32 accumulation (here FP64,
the difference is the accumulation order only), exact GELU, MSE loss over the
85 real outputs, bias gradients summed from the FP32 activation gradients.
"""
from __future__ import annotations

import math

import numpy as np

N_IN, N_IN_PAD, N_H, N_OUT, N_OUT_PAD = 397, 400, 256, 85, 96
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_H * N_IN_PAD
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_OUT_PAD * N_H
N_PARAMS = OFF_B3 + N_OUT_PAD


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).copy()
    b = a.view(np.uint32)
    b += ((b >> 16) & 1) + np.uint32(0x7FFF)
    b &= np.uint32(0xFFFF0000)
    return a.astype(np.float64)


def _erf(x):
    return np.vectorize(math.erf)(x)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    W1 = P[OFF_W1:OFF_B1].reshape(N_H, N_IN_PAD)
    b1 = P[OFF_B1:OFF_W2]
    W2 = P[OFF_W2:OFF_B2].reshape(N_H, N_H)
    b2 = P[OFF_B2:OFF_W3]
    W3 = P[OFF_W3:OFF_B3].reshape(N_OUT_PAD, N_H)
    b3 = P[OFF_B3:]
    return W1, b1, W2, b2, W3, b3


def forward(P, X, round_bf16=True):
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(P)
    Xp = np.zeros((X.shape[0], N_IN_PAD))
    Xp[:, :N_IN] = X
    Xb = r(Xp)
    pre1 = Xb @ r(W1).T + b1
    H1 = r(gelu(pre1))
    pre2 = H1 @ r(W2).T + b2
    H2 = r(gelu(pre2))
    Y = H2 @ r(W3).T + b3
    return Y[:, :N_OUT], (Xb, pre1, H1, pre2, H2, Y)


def loss_grad(P, X, T, round_bf16=True):
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(P)
    M = X.shape[0]
    Y, (Xb, pre1, H1, pre2, H2, Yfull) = forward(P, X, round_bf16)
    E = Y - T
    loss = float((E ** 2).sum() / (M * N_OUT))
    dY = np.zeros((M, N_OUT_PAD))
    dY[:, :N_OUT] = 2.0 * E / (M * N_OUT)
    if round_bf16:
        dY = dY.astype(np.float32).astype(np.float64)
    dYb = r(dY)
    G = np.zeros(N_PARAMS)
    gW3 = dYb.T @ H2
    gb3 = dY.sum(0)
    dH2 = dYb @ r(W3)
    dA2 = dH2 * gelu_grad(pre2)
    dA2b = r(dA2)
    gW2 = dA2b.T @ H1
    gb2 = dA2.sum(0)
    dH1 = dA2b @ r(W2)
    dA1 = dH1 * gelu_grad(pre1)
    dA1b = r(dA1)
    gW1 = dA1b.T @ Xb
    gb1 = dA1.sum(0)
    gW1[:, N_IN:] = 0.0
    gW3[N_OUT:, :] = 0.0
    gb3[N_OUT:] = 0.0
    G[OFF_W1:OFF_B1] = gW1.ravel()
    G[OFF_B1:OFF_W2] = gb1
    G[OFF_W2:OFF_B2] = gW2.ravel()
    G[OFF_B2:OFF_W3] = gb2
    G[OFF_W3:OFF_B3] = gW3.ravel()
    G[OFF_B3:] = gb3
    return loss, G


def loss_only_fp64(P, X, T):
    """Loss without any rounding (for finite-difference checks of loss_grad's
    structure on the CPU)."""
    W1, b1, W2, b2, W3, b3 = unpack(P)
    Xp = np.zeros((X.shape[0], N_IN_PAD))
    Xp[:, :N_IN] = X
    H1 = gelu(Xp @ W1.T + b1)
    H2 = gelu(H1 @ W2.T + b2)
    Y = (H2 @ W3.T + b3)[:, :N_OUT]
    return float(((Y - T) ** 2).sum() / (X.shape[0] * N_OUT))
