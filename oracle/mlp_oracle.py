"""FP64 reference of the surrogate MLP -- TEST INFRASTRUCTURE ONLY.

Forward and backward of the 12 -> 4 x 256 (GELU) -> 10 network in float64
numpy, with the inputs and weights rounded to BF16 exactly as the device
kernels round them, and GELU in the same tanh form (evaluated exactly
here, with the special-function tanh on the device).  Used to check the
device's tensor-core forward, backward and parameter gradients.
"""
import math

import numpy as np

NL = 5


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


# GELU in the tanh form of Hendrycks and Gimpel (2016), the form the
# library's kernels evaluate: 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))
_C0 = math.sqrt(2.0 / math.pi)
_C1 = _C0 * 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(z * (_C0 + _C1 * z * z)))


def gelu_grad(z):
    z2 = z * z
    t = np.tanh(z * (_C0 + _C1 * z2))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * (_C0 + 3.0 * _C1 * z2)


def forward(W, b, x, rounding=True):
    """x: (M, 12) normalised inputs.  Returns output (M, 10) and the cache.
    rounding=False evaluates the same network in plain float64 (for
    finite-difference checks of the analytic gradients)."""
    rnd = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    a = np.zeros((len(x), W[0].shape[0]))
    a[:, :x.shape[1]] = rnd(x)
    acts, zs = [a], []
    for l in range(NL):
        z = acts[-1] @ rnd(W[l]) + np.asarray(b[l], dtype=np.float64)
        zs.append(z)
        if l < NL - 1:
            acts.append(rnd(gelu(z)))
    return zs[-1][:, :10], (acts, zs)


def loss_and_grads(W, b, x, t, rounding=True):
    """MSE over the 10 outputs and its parameter gradients (float64)."""
    rnd = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    out, (acts, zs) = forward(W, b, x, rounding)
    M = len(x)
    d = out - t
    loss = float((d * d).mean())
    dz = np.zeros_like(zs[-1])
    dz[:, :10] = 2.0 * d / (M * 10)
    gW, gb = [None] * NL, [None] * NL
    for l in range(NL - 1, -1, -1):
        gW[l] = acts[l].T @ dz
        gb[l] = dz.sum(axis=0)
        if l == 0:
            break
        da = dz @ rnd(W[l]).T
        dz = da * gelu_grad(zs[l - 1])
    return loss, gW, gb
