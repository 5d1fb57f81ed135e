"""FP64 restatement of the warm-start network -- TEST INFRASTRUCTURE ONLY.

Checks the tensor-core forward pass and the CUDA-core backward pass of
splishsplash_gb300/csrc/mlp.cu.  It emulates the BF16 roundings the device path
applies (inputs, weights, post-GELU activations: round to nearest even) and does
all arithmetic in FP64, so the remaining differences are the device's FP32
accumulation order.  Parameter layout (row-major): W1[64][16] b1[64] W2[64][64]
b2[64] W3[8][64] b3[8]; 10 inputs, 2 outputs used.
"""
import numpy as np
from scipy.special import erf

N_IN, N_IN_PAD, N_H, N_OUT, N_OUT_PAD = 10, 16, 64, 2, 8
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_H * N_IN_PAD
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_OUT_PAD * N_H
N_PARAMS = OFF_B3 + N_OUT_PAD


def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float32)
    W1 = p[OFF_W1:OFF_B1].reshape(N_H, N_IN_PAD)[:, :N_IN]
    b1 = p[OFF_B1:OFF_W2].astype(np.float64)
    W2 = p[OFF_W2:OFF_B2].reshape(N_H, N_H)
    b2 = p[OFF_B2:OFF_W3].astype(np.float64)
    W3 = p[OFF_W3:OFF_B3].reshape(N_OUT_PAD, N_H)[:N_OUT]
    b3 = p[OFF_B3:OFF_B3 + N_OUT].astype(np.float64)
    return bf16(W1), b1, bf16(W2), b2, bf16(W3), b3


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    Xb = bf16(X)
    Z1 = Xb @ W1.T + b1
    H1 = bf16(gelu(Z1))
    Z2 = H1 @ W2.T + b2
    H2 = bf16(gelu(Z2))
    Y = H2 @ W3.T + b3
    return Y, (Xb, Z1, H1, Z2, H2)


def loss_grad(p, X, T, mask=None):
    """Mean over samples of sum_o mask (y - t)^2 and its gradient in the device layout."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    Y, (Xb, Z1, H1, Z2, H2) = forward(p, X)
    n = X.shape[0]
    M = np.ones_like(Y) if mask is None else np.asarray(mask, np.float64)
    D = Y - np.asarray(T, np.float64)
    loss = float(np.sum(M * D * D) / n)
    dY = 2.0 * M * D / n
    g = np.zeros(N_PARAMS)
    gW3 = np.zeros((N_OUT_PAD, N_H))
    gW3[:N_OUT] = dY.T @ H2
    g[OFF_W3:OFF_B3] = gW3.ravel()
    g[OFF_B3:OFF_B3 + N_OUT] = dY.sum(0)
    dZ2 = (dY @ W3) * gelu_grad(Z2)
    g[OFF_W2:OFF_B2] = (dZ2.T @ H1).ravel()
    g[OFF_B2:OFF_W3] = dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * gelu_grad(Z1)
    gW1 = np.zeros((N_H, N_IN_PAD))
    gW1[:, :N_IN] = dZ1.T @ Xb
    g[OFF_W1:OFF_B1] = gW1.ravel()
    g[OFF_B1:OFF_W2] = dZ1.sum(0)
    return loss, g
