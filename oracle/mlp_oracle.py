"""CPU oracle of the learned warm start's network (test infrastructure only).

The warm-start network has no counterpart in the reference: EPSpectral.jl takes a caller's
`Σ_init` (src/scgd0.jl:66, 204-212) and this project proposes one with a multilayer perceptron.
This module restates, in NumPy FP64, the exact arithmetic that the GPU kernels of the warm start
perform, so that the tests can check the GPU forward pass, loss, gradients and Adam steps:

* layers d_0 -> ... -> d_L, z_l = x_l W_l^T + b_l, x_{l+1} = SiLU(z_l) = z_l / (1 + e^{-z_l})
  between layers, linear output;
* the products use the weights rounded to BF16 (round to nearest even), as the kernels do; the
  gradients are those of the rounded network (straight-through for the rounding);
* loss = mean over rows and outputs of (y_pred - y)^2;
* Adam: m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2, w -= lr (m / (1-b1^t)) / (sqrt(v / (1-b2^t)) + eps).

Parameters are one flat vector: per layer W_l [d_{l+1}][d_l] row-major, then b_l [d_{l+1}].
Only the tests, the smoke check and the benchmark's CPU leg import this file.
"""
from __future__ import annotations

import numpy as np


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unflatten(params: np.ndarray, dims) -> list[tuple[np.ndarray, np.ndarray]]:
    out, off = [], 0
    for din, dout in zip(dims[:-1], dims[1:]):
        W = np.asarray(params[off:off + din * dout], dtype=np.float64).reshape(dout, din)
        off += din * dout
        b = np.asarray(params[off:off + dout], dtype=np.float64)
        off += dout
        out.append((W, b))
    if off != len(params):
        raise ValueError(f"{len(params)} parameters for layer widths {list(dims)} (expected {off})")
    return out


def nparams(dims) -> int:
    return int(sum(a * b + b for a, b in zip(dims[:-1], dims[1:])))


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, dims, X, *, round_bf16=True):
    """Returns the output and the per-layer (input, pre-activation) pairs."""
    layers = unflatten(params, dims)
    x = np.asarray(X, dtype=np.float64)
    cache = []
    for l, (W, b) in enumerate(layers):
        Wq = bf16_round(W) if round_bf16 else W
        z = x @ Wq.T + b
        cache.append((x, z, Wq))
        x = _silu(z) if l + 1 < len(layers) else z
    return x, cache


def predict(params, dims, X, *, round_bf16=True):
    return forward(params, dims, X, round_bf16=round_bf16)[0]


def loss_and_grad(params, dims, X, Y, *, round_bf16=True):
    """Mean squared error and its gradient, flat like `params`."""
    P, cache = forward(params, dims, X, round_bf16=round_bf16)
    Y = np.asarray(Y, dtype=np.float64)
    n, d = Y.shape
    E = P - Y
    loss = float(np.sum(E * E) / (n * d))
    dz = 2.0 * E / (n * d)
    grads = [None] * len(cache)
    for l in range(len(cache) - 1, -1, -1):
        x, z, Wq = cache[l]
        gW = dz.T @ x
        gb = dz.sum(axis=0)
        grads[l] = (gW, gb)
        if l > 0:
            dx = dz @ Wq
            dz = dx * _silu_grad(cache[l - 1][1])
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def adam_step(params, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (t counts from 1); returns the new (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    c1, c2 = 1 - b1 ** t, 1 - b2 ** t
    return params - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def train(params, dims, X, Y, *, epochs, batch, lr, perm=None):
    """Minibatch Adam as epsp_warmstart_train: each minibatch's loss is its own mean."""
    p = np.asarray(params, dtype=np.float64).copy()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    n = len(X)
    t = 0
    hist = []
    for e in range(epochs):
        order = np.arange(n) if perm is None else np.asarray(perm[e])
        tot = 0.0
        for r0 in range(0, n, batch):
            idx = order[r0:r0 + batch]
            loss, g = loss_and_grad(p, dims, X[idx], Y[idx])
            tot += loss * len(idx) * Y.shape[1]
            t += 1
            p, m, v = adam_step(p, g, m, v, t, lr)
        hist.append(tot / (n * Y.shape[1]))
    return p, np.array(hist)
