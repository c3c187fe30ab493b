"""CPU oracle of the learned-initial-iterate network (test infrastructure only).

Restates, in numpy with float64 accumulation, what the device network computes:
operands rounded to bfloat16 (round to nearest even) exactly where the device
rounds them, products accumulated in high precision, ReLU on hidden layers, a
linear output layer, the mean-squared-error loss and its gradients, and the Adam
update.  The device accumulates in FP32, so device and oracle agree to FP32
rounding of the sums, plus an occasional one-ulp bfloat16 flip of an activation
whose FP32 value sits on a rounding boundary.

There is no counterpart of this network in the reference; the parameter layout
(W0 [in x out] row-major, b0, W1, b1, ...) is the one of vfvm_mlp_params.
"""
from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unflatten(theta: np.ndarray, sizes):
    """[(W, b)] per layer from the flat parameter vector."""
    out, off = [], 0
    for k, n in zip(sizes[:-1], sizes[1:]):
        W = theta[off:off + k * n].reshape(k, n)
        off += k * n
        b = theta[off:off + n]
        off += n
        out.append((W, b))
    assert off == theta.size
    return out


def _rounder(exact: bool):
    if exact:
        return lambda a: np.asarray(a, dtype=np.float64)
    return lambda a: bf16(np.asarray(a, dtype=np.float32)).astype(np.float64)


def forward(theta, sizes, X, exact: bool = False):
    """Returns (Y, cache) with Y the float64 output of the network on X.
    exact=True skips every rounding (float64 throughout): the plain network,
    used to check the backward formulas against finite differences."""
    rd = _rounder(exact)
    layers = unflatten(np.asarray(theta, dtype=np.float64 if exact else np.float32), sizes)
    xb = rd(X)
    cache = []
    for l, (W, b) in enumerate(layers):
        Wb = rd(W)
        Z = xb @ Wb + np.asarray(b, dtype=np.float64)
        last = l + 1 == len(layers)
        A = Z if last else np.maximum(Z, 0.0)
        cache.append((xb, Wb, Z))
        xb = rd(A)
    return Z, cache


def loss_and_gradients(theta, sizes, X, T, exact: bool = False):
    """Mean squared error of net(X) against T and its gradient (flat, float64)."""
    rd = _rounder(exact)
    Y, cache = forward(theta, sizes, X, exact)
    B, n = T.shape
    E = Y - T
    loss = float(np.mean(E * E))
    dA = 2.0 * E / (B * n)
    if not exact:
        dA = dA.astype(np.float32).astype(np.float64)
    grads = []
    for l in range(len(cache) - 1, -1, -1):
        xb, Wb, Z = cache[l]
        dZ = dA if l + 1 == len(cache) else np.where(Z > 0.0, dA, 0.0)
        dZb = rd(dZ)
        gW = xb.T @ dZb
        gb = dZ.sum(axis=0)
        grads.append((gW, gb))
        dA = dZb @ Wb.T
    flat = []
    for gW, gb in reversed(grads):
        flat.append(gW.ravel())
        flat.append(gb)
    return loss, np.concatenate(flat)


def adam(theta, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected), returns (theta, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
