"""CPU oracle of the eigen-interval network (test infrastructure only).

A numpy restatement of the forward and backward passes that the library's
tensor-core kernels implement (include/ggem_surrogate.h): standardised
inputs, BF16 operands of every matrix product (round to nearest even), FP32
accumulation, FP32 bias and SiLU, BF16 activations, FP32 output layer;
loss = mean over rows of the summed squared error of the two standardised
outputs.  The parameter layout is the library's flat vector
(W1^T [128 x 48], b1, W2^T, b2, W3^T, b3, W4^T [128 x 128], b4).

This network has no counterpart in the reference (it replaces the SLEPc
eigenvalue estimate of brownian_system.C:527-657); the oracle pins the
library's own arithmetic so that the GPU gradients can be checked.
"""
from __future__ import annotations

import numpy as np

IN, IN_PAD, HID, OUT = 35, 48, 128, 2
IN_DIMS = (IN_PAD, HID, HID, HID)


def bf16(a) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(params: np.ndarray):
    """[(W^T [128 x in], b [128])] for the four layers."""
    out, o = [], 0
    for d in IN_DIMS:
        wt = params[o:o + HID * d].reshape(HID, d)
        o += HID * d
        b = params[o:o + HID]
        o += HID
        out.append((wt, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _arith(exact):
    """(dtype, rounding of product operands): the device's BF16/FP32 mix, or
    exact float64 arithmetic for finite-difference checks of the formulas."""
    if exact:
        return np.float64, (lambda a: np.asarray(a, np.float64))
    return np.float32, bf16


def stage(X, norm, exact=False):
    dt, r = _arith(exact)
    mean, sd = norm[:IN], norm[IN:2 * IN]
    inv = np.where(sd > 0, 1.0 / np.where(sd > 0, sd, 1.0), 1.0).astype(dt)
    x = ((np.asarray(X, dt) - mean.astype(dt)) * inv).astype(dt)
    xp = np.zeros((len(x), IN_PAD), dt)
    xp[:, :IN] = x
    return r(xp)


def forward(params, norm, X, exact=False):
    """Standardised outputs [n x 2] and the cache of the backward pass."""
    dt, r = _arith(exact)
    layers = unpack(np.asarray(params, dt))
    h = stage(X, norm, exact)
    cache = [h]
    zs = []
    for l, (wt, b) in enumerate(layers):
        z = (h @ r(wt).T).astype(dt) + b
        zs.append(z)
        if l < 3:
            h = r(silu(z).astype(dt))
            cache.append(h)
    y = zs[-1][:, :OUT]
    return y, (cache, zs, layers)


def loss_and_grad(params, norm, X, Y, exact=False):
    """Loss and gradient (flat, the parameter layout) for raw targets Y."""
    dt, r = _arith(exact)
    y, (cache, zs, layers) = forward(params, norm, X, exact)
    ym, ysd = norm[2 * IN:2 * IN + OUT], norm[2 * IN + OUT:]
    t = ((np.asarray(Y, dt) - ym) / np.where(ysd > 0, ysd, 1.0)).astype(dt)
    n = len(X)
    e = y - t
    loss = float((e * e).sum() / n)
    dz = np.zeros((n, HID), dt)
    dz[:, :OUT] = 2.0 * e / n
    grads = [None] * 4
    for l in range(3, -1, -1):
        wt, _ = layers[l]
        dzb = r(dz)
        gw = (dzb.T @ cache[l]).astype(dt)
        gb = dz.sum(axis=0).astype(dt)
        grads[l] = (gw, gb)
        if l == 0:
            break
        dh = (dzb @ r(wt)).astype(dt)
        dz = (dh * dsilu(zs[l - 1])).astype(dt)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat


def predict(params, norm, X):
    y, _ = forward(params, norm, X)
    ym, ysd = norm[2 * IN:2 * IN + OUT], norm[2 * IN + OUT:]
    return y * ysd + ym
