"""CPU check of the surrogate MLP -- TEST INFRASTRUCTURE.

FP64 numpy forward and backward of the same network on the same BF16-rounded operands as the
GPU kernels (weights, inputs, hidden activations and output deltas rounded to BF16, every
product accumulated exactly), so that the gradients can be compared to FP32 round-off.
"""
import numpy as np


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(layers, x):
    """layers: [(W, b)] FP32; returns the pre-activations and the BF16 activations."""
    a = [bf16(x)]
    zs = []
    for l, (W, b) in enumerate(layers):
        z = a[-1] @ bf16(W).T + np.asarray(b, np.float64)
        zs.append(z)
        if l + 1 < len(layers):
            a.append(bf16(silu(z)))
    return zs, a


def grads(layers, x, t):
    """Gradients of (1/2B) sum (y - t)^2 with the GPU's rounding points."""
    B = x.shape[0]
    zs, a = forward(layers, x)
    d = (zs[-1] - t) / B
    loss = 0.5 * np.sum((zs[-1] - t) ** 2) / B
    out = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        db = bf16(d)
        gW = db.T @ a[l]
        gb = d.sum(0)
        out[l] = (gW, gb)
        if l > 0:
            da = db @ bf16(layers[l][0])
            z = zs[l - 1]
            s = 1.0 / (1.0 + np.exp(-z))
            d = da * (s * (1.0 + z * (1.0 - s)))
    return loss, out


def grads_exact(layers, x, t):
    """The same gradients without BF16 rounding (FP64 throughout), for finite-difference checks."""
    B = x.shape[0]
    a = [np.asarray(x, np.float64)]
    zs = []
    for l, (W, b) in enumerate(layers):
        z = a[-1] @ np.asarray(W, np.float64).T + np.asarray(b, np.float64)
        zs.append(z)
        if l + 1 < len(layers):
            a.append(silu(z))
    loss = 0.5 * np.sum((zs[-1] - t) ** 2) / B
    d = (zs[-1] - t) / B
    out = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        out[l] = (d.T @ a[l], d.sum(0))
        if l > 0:
            z = zs[l - 1]
            s = 1.0 / (1.0 + np.exp(-z))
            d = (d @ np.asarray(layers[l][0], np.float64)) * (s * (1.0 + z * (1.0 - s)))
    return loss, out
