"""ORACLE — test infrastructure only: a numpy restatement of the learned far
field's network (baby_shark_gb300/csrc/mlp.cu) for checking the GPU's
forward pass and gradients.  The learned stage has no counterpart in the
reference crate, so this is the CPU check of this repository's own method.

The GPU computes in BF16 on the tensor cores with FP32 accumulation; the
restatement rounds the same intermediate values to BF16 (round to nearest
even) and accumulates in float64, so the two differ only by FP32 summation
order and the GPU's fast exponential.
"""
import numpy as np

OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3, NP = 0, 4096, 4160, 8256, 8320, 8384, 8385


ROUND = True  # False: no BF16 rounding (for finite-difference checks of the restatement itself)


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    if not ROUND:
        return np.asarray(x, np.float64)
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(params):
    p = np.asarray(params, np.float32 if ROUND else np.float64)
    return (p[OFF_W1:OFF_B1].reshape(64, 64), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(64, 64),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def features(points, freq, centre, scale):
    xn = ((np.asarray(points, np.float32) - np.asarray(centre, np.float32)) * np.float32(scale)).astype(np.float64)
    v = xn @ np.asarray(freq, np.float64).reshape(32, 3).T
    f = np.concatenate([np.sin(np.pi * v), np.cos(np.pi * v)], axis=1)
    return bf16(f if not ROUND else f.astype(np.float32)).astype(np.float64)


def forward(params, freq, centre, scale, points):
    """Returns (y, cache) for the points (n, 3)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    F = features(points, freq, centre, scale)
    z1 = F @ bf16(W1).astype(np.float64) + b1
    h1 = bf16(silu(z1) if not ROUND else silu(z1).astype(np.float32)).astype(np.float64)
    z2 = h1 @ bf16(W2).astype(np.float64) + b2
    h2 = silu(z2)
    y = h2 @ w3.astype(np.float64) + float(b3)
    return y, (F, z1, h1, z2, h2)


def gradients(params, freq, centre, scale, points, targets):
    """Mean squared error and its gradient w.r.t. the 8385 parameters, with
    the GPU's BF16 roundings of features, activations and pre-activation
    gradients."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    y, (F, z1, h1, z2, h2) = forward(params, freq, centre, scale, points)
    n = len(y)
    e = y - np.asarray(targets, np.float64)
    dy = 2.0 * e / n
    g = np.zeros(NP)
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    dz2 = dy[:, None] * w3.astype(np.float64)[None, :] * dsilu(z2)
    dz2 = bf16(dz2 if not ROUND else dz2.astype(np.float32)).astype(np.float64)
    dh1 = dz2 @ bf16(W2).astype(np.float64).T
    dz1 = dh1 * dsilu(z1)
    dz1 = bf16(dz1 if not ROUND else dz1.astype(np.float32)).astype(np.float64)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0)
    g[OFF_W1:OFF_B1] = (F.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0)
    return float(np.mean(e * e)), g
