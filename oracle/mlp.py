"""FP64 CPU oracle of the warm-start MLP -- TEST INFRASTRUCTURE ONLY.

The reference has no learned component; this restates, in numpy float64, the network the
GPU kernels train and run, so their forward pass, gradients and optimiser step can be
checked: two hidden ReLU layers, MSE loss, Adam (Kingma & Ba 2015).

Parameter layout (the device buffer's): W1 [H][Din], b1 [H], W2 [H][H], b2 [H], W3 [Dout][H], b3 [Dout].
"""
from __future__ import annotations

import numpy as np


def sizes(din: int, h: int, dout: int):
    return [(h, din), (h,), (h, h), (h,), (dout, h), (dout,)]


def unpack(theta: np.ndarray, din: int, h: int, dout: int):
    out, o = [], 0
    for s in sizes(din, h, dout):
        n = int(np.prod(s))
        out.append(theta[o:o + n].reshape(s))
        o += n
    return out


def nparams(din: int, h: int, dout: int) -> int:
    return sum(int(np.prod(s)) for s in sizes(din, h, dout))


def init(din: int, h: int, dout: int, seed: int) -> np.ndarray:
    """He-uniform weights from a counter hash, zero biases (same values as the device init)."""
    theta = np.zeros(nparams(din, h, dout))
    o = 0
    for s in sizes(din, h, dout):
        n = int(np.prod(s))
        if len(s) == 2:
            bound = np.sqrt(6.0 / s[1])
            u = np.array([hash_uniform(seed, o + j) for j in range(n)])
            theta[o:o + n] = (2.0 * u - 1.0) * bound
        o += n
    return theta


def hash_uniform(seed: int, i: int) -> float:
    """U[0,1) from a splitmix64 mix of (seed, i) -- the device uses the same 24 bits."""
    M = (1 << 64) - 1
    z = (seed * 0x9E3779B97F4A7C15 + (i + 1) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    z ^= z >> 31
    return (z >> 40) / float(1 << 24)


def forward(theta, X, din, h, dout):
    W1, b1, W2, b2, W3, b3 = unpack(theta, din, h, dout)
    z1 = X @ W1.T + b1
    a1 = np.maximum(z1, 0.0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0.0)
    y = a2 @ W3.T + b3
    return y, (X, z1, a1, z2, a2)


def loss_and_grad(theta, X, T, din, h, dout):
    """loss = sum over the batch of 0.5 * ||y - t||^2 / (B * dout); gradient in the layout."""
    W1, b1, W2, b2, W3, b3 = unpack(theta, din, h, dout)
    y, (X, z1, a1, z2, a2) = forward(theta, X, din, h, dout)
    B = X.shape[0]
    d = (y - T) / (B * dout)
    loss = 0.5 * float(((y - T) ** 2).sum()) / (B * dout)
    gW3 = d.T @ a2
    gb3 = d.sum(0)
    d2 = (d @ W3) * (z2 > 0)
    gW2 = d2.T @ a1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (z1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def adam_step(theta, m, v, g, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
