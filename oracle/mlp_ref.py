"""NumPy FP64 reference of the learned screen's MLP (TEST INFRASTRUCTURE ONLY: the checker of the CUDA training and
inference kernels).  Same parameter layout and the same BF16 roundings as the kernels: BF16 inputs and weights of
the three hidden layers, BF16 activations fed to layers 2 and 3, FP32 biases and head, tanh-form GELU."""
from __future__ import annotations

import numpy as np

NIN, NH = 16, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NIN
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH * NH
OFF_W4 = OFF_B3 + NH
OFF_B4 = OFF_W4 + NH
NPARAM = OFF_B4 + 1


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    k0, k1 = 0.7978845608028654, 0.044715
    return 0.5 * x * (1.0 + np.tanh(k0 * (x + k1 * x ** 3)))


def gelu_grad(x):
    k0, k1 = 0.7978845608028654, 0.044715
    t = np.tanh(k0 * (x + k1 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * k0 * (1 + 3 * k1 * x * x)


def unpack(p, rounded=True):
    r = bf16 if rounded else (lambda a: np.asarray(a, dtype=np.float64))
    W1 = r(p[OFF_W1:OFF_B1]).reshape(NH, NIN)
    W2 = r(p[OFF_W2:OFF_B2]).reshape(NH, NH)
    W3 = r(p[OFF_W3:OFF_B3]).reshape(NH, NH)
    return (W1, np.asarray(p[OFF_B1:OFF_W2], np.float64), W2, np.asarray(p[OFF_B2:OFF_W3], np.float64), W3,
            np.asarray(p[OFF_B3:OFF_W4], np.float64), np.asarray(p[OFF_W4:OFF_B4], np.float64), float(p[OFF_B4]))


def forward(X, p, rounded=True):
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p, rounded)
    X = bf16(X) if rounded else np.asarray(X, np.float64)
    rb = bf16 if rounded else (lambda a: a)
    z1 = X @ W1.T + b1
    h1 = rb(gelu(z1))
    z2 = h1 @ W2.T + b2
    h2 = rb(gelu(z2))
    z3 = h2 @ W3.T + b3
    h3 = gelu(z3)
    return h3 @ w4 + b4, (X, z1, h1, z2, h2, z3, h3)


def grad(X, y, p, rounded=True):
    """Gradient of 0.5 sum (f - y)^2 (straight-through the BF16 roundings, as the kernels do)."""
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p, rounded)
    out, (Xr, z1, h1, z2, h2, z3, h3) = forward(X, p, rounded)
    dy = out - y
    g = np.zeros(NPARAM)
    g[OFF_W4:OFF_B4] = h3.T @ dy
    g[OFF_B4] = dy.sum()
    d3 = (dy[:, None] * w4[None, :]) * gelu_grad(z3)
    g[OFF_W3:OFF_B3] = (d3.T @ h2).ravel()
    g[OFF_B3:OFF_W4] = d3.sum(0)
    d2 = (d3 @ W3) * gelu_grad(z2)
    g[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(0)
    d1 = (d2 @ W2) * gelu_grad(z1)
    g[OFF_W1:OFF_B1] = (d1.T @ Xr).ravel()
    g[OFF_B1:OFF_W2] = d1.sum(0)
    return g, 0.5 * float((dy ** 2).sum())


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM)
    p[OFF_W1:OFF_B1] = rng.standard_normal(NH * NIN) * np.sqrt(2.0 / 14)
    p[OFF_W2:OFF_B2] = rng.standard_normal(NH * NH) * np.sqrt(2.0 / NH)
    p[OFF_W3:OFF_B3] = rng.standard_normal(NH * NH) * np.sqrt(2.0 / NH)
    p[OFF_W4:OFF_B4] = rng.standard_normal(NH) * np.sqrt(1.0 / NH)
    return p
