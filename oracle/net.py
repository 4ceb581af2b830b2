"""CPU restatement of the learned closure network -- TEST INFRASTRUCTURE ONLY.

What the CUDA training and inference kernels (gradients, forward outputs) of
the learned-closure form are compared with: a 3-D convolutional net on the LES grid
with periodic 3x3x3 kernels, channels 3 -> 32 -> 32 -> 3 and GELU after the
first two layers (no counterpart in the reference; its closures are the
exact and classic ones of ``src/N.jl:1137-1226``).

Tensors are channel-last ``[b, z, y, x, c]`` float64; weights are
``W[tap, ci, co]`` with ``tap = (dz+1)*9 + (dy+1)*3 + (dx+1)`` and biases
``b[co]``; a layer computes
``pre[v, co] = b[co] + sum_{tap, ci} x[v + tap, ci] W[tap, ci, co]``
with periodic wrap.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def shift(x: np.ndarray, dz: int, dy: int, dx: int) -> np.ndarray:
    """``shift(x)[v] = x[v + (dz, dy, dx)]`` periodically ([b, z, y, x, c])."""
    return np.roll(x, (-dz, -dy, -dx), axis=(1, 2, 3))


def conv(x, W, b):
    out = np.zeros(x.shape[:4] + (W.shape[2],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += shift(x, dz, dy, dx) @ W[t]
    return out + b


def conv_backward(x, W, dout):
    """Gradients of ``conv`` w.r.t. its input, weights and bias."""
    dx = np.zeros_like(x)
    dW = np.zeros_like(W)
    for t, (dz, dy, dx_) in enumerate(TAPS):
        xs = shift(x, dz, dy, dx_)
        dW[t] = np.einsum("bzyxi,bzyxo->io", xs, dout, optimize=True)
        dx += shift(dout @ W[t].T, -dz, -dy, -dx_)
    db = dout.sum(axis=(0, 1, 2, 3))
    return dx, dW, db


def gelu(x):
    return 0.5 * x * (1 + erf(x / math.sqrt(2)))


def gelu_grad(x):
    return 0.5 * (1 + erf(x / math.sqrt(2))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def init_params(seed: int, hidden: int = 32, cin: int = 3, cout: int = 3):
    """He-style initialisation, for tests only (the device draws its own)."""
    rng = np.random.default_rng(seed)
    dims = [(cin, hidden), (hidden, hidden), (hidden, cout)]
    params = []
    for ci, co in dims:
        std = math.sqrt(2.0 / (27 * ci))
        params.append((rng.normal(0, std, (27, ci, co)), np.zeros(co)))
    return params


def forward(params, x):
    """Returns the output and the cache of pre-activations and inputs."""
    cache = []
    h = x
    for li, (W, b) in enumerate(params):
        pre = conv(h, W, b)
        cache.append((h, pre))
        h = gelu(pre) if li < len(params) - 1 else pre
    return h, cache


def loss_and_grads(params, x, target):
    """MSE loss ``mean((f(x) - target)^2)`` and its parameter gradients."""
    out, cache = forward(params, x)
    diff = out - target
    loss = float(np.mean(diff * diff))
    g = 2.0 * diff / diff.size
    grads = [None] * len(params)
    for li in range(len(params) - 1, -1, -1):
        h, pre = cache[li]
        if li < len(params) - 1:
            g = g * gelu_grad(pre)
        dx, dW, db = conv_backward(h, params[li][0], g)
        grads[li] = (dW, db)
        g = dx
    return loss, grads


def adam_step(params, grads, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015) with bias correction."""
    state["t"] = state.get("t", 0) + 1
    t = state["t"]
    new = []
    for i, ((W, b), (gW, gb)) in enumerate(zip(params, grads)):
        out = []
        for j, (p, gp) in enumerate(((W, gW), (b, gb))):
            m = state.setdefault(("m", i, j), np.zeros_like(p))
            v = state.setdefault(("v", i, j), np.zeros_like(p))
            m[...] = b1 * m + (1 - b1) * gp
            v[...] = b2 * v + (1 - b2) * gp * gp
            mh = m / (1 - b1**t)
            vh = v / (1 - b2**t)
            out.append(p - lr * mh / (np.sqrt(vh) + eps))
        new.append(tuple(out))
    return new
