"""CPU oracle of the quadrature-order selector network (test infrastructure
only): forward pass, mean softmax cross-entropy and its analytic gradient for
the 24-64-64-5 ReLU network with the flat parameter layout
W1 (24 x 64, row-major), b1, W2 (64 x 64), b2, W3 (64 x 5), b3, in float64;
plus a central-difference gradient that pins the analytic one.

The network has no counterpart in the reference (which always integrates with
its fixed 16-point rule, boundaryelementsolver.cpp:857-893); the oracle states
the mathematics the GPU training kernels must reproduce."""
from __future__ import annotations

import numpy as np

NF, H, C = 24, 64, 5
SHAPES = [("W1", (NF, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, C)),
          ("b3", (C,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    p = np.asarray(p, np.float64)
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    return out


def init(seed=0):
    rng = np.random.default_rng(seed)
    parts = []
    for name, shp in SHAPES:
        if name.startswith("W"):
            parts.append(rng.standard_normal(shp).ravel() * np.sqrt(2.0 / shp[0]))
        else:
            parts.append(np.zeros(shp))
    return np.concatenate(parts)


def forward(p, X):
    w = unpack(p)
    X = np.asarray(X, np.float64)
    z1 = X @ w["W1"] + w["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ w["W2"] + w["b2"]
    h2 = np.maximum(z2, 0)
    return h2 @ w["W3"] + w["b3"], (X, z1, h1, z2, h2)


def loss(p, X, y):
    z, _ = forward(p, X)
    zm = z.max(1, keepdims=True)
    lse = np.log(np.exp(z - zm).sum(1)) + zm[:, 0]
    return float(np.mean(lse - z[np.arange(len(y)), y]))


def grad(p, X, y):
    """Analytic gradient of the mean cross-entropy (backpropagation)."""
    w = unpack(p)
    z, (X, z1, h1, z2, h2) = forward(p, X)
    B = len(y)
    e = np.exp(z - z.max(1, keepdims=True))
    P = e / e.sum(1, keepdims=True)
    d3 = P.copy()
    d3[np.arange(B), y] -= 1.0
    d3 /= B
    d2 = (d3 @ w["W3"].T) * (z2 > 0)
    d1 = (d2 @ w["W2"].T) * (z1 > 0)
    g = {"W1": X.T @ d1, "b1": d1.sum(0), "W2": h1.T @ d2, "b2": d2.sum(0),
         "W3": h2.T @ d3, "b3": d3.sum(0)}
    return np.concatenate([g[name].ravel() for name, _ in SHAPES])


def grad_fd(p, X, y, idx, eps=1e-6):
    """Central differences of the loss for the parameters in idx."""
    p = np.asarray(p, np.float64)
    out = np.zeros(len(idx))
    for t, i in enumerate(idx):
        a = p.copy()
        b = p.copy()
        a[i] += eps
        b[i] -= eps
        out[t] = (loss(a, X, y) - loss(b, X, y)) / (2 * eps)
    return out


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)
