"""NumPy restatement of the point-cloud warm-start network (test infrastructure).

It has no reference counterpart (the reference has no learned warm start).
It is the CPU oracle of the GPU kernels in electrodrive_gb300/csrc/pcn.cu:
the same parameter layout, features, forward pass, loss and backward pass.
With ``emulate_bf16=True`` the values are rounded to BF16 at the same points
as the kernels: the inputs, the weights of the three per-panel layers, the
stored activations and the backpropagated pre-activation gradients.  Those
results are then comparable with the kernels' FP32-accumulated ones.  With
``emulate_bf16=False`` it is the exact FP64 network, and finite differences
check its gradients.
"""
from __future__ import annotations

import numpy as np

WIDTH = 128
INPUTS = 16
_SHAPES = [("W1", (WIDTH, INPUTS)), ("b1", (WIDTH,)), ("W2", (WIDTH, WIDTH)), ("V2", (WIDTH, WIDTH)),
           ("b2", (WIDTH,)), ("W3", (WIDTH, WIDTH)), ("b3", (WIDTH,)), ("w4", (WIDTH,)), ("b4", (1,))]
NPARAMS = sum(int(np.prod(s)) for _, s in _SHAPES)


def unpack(theta):
    out, o = {}, 0
    for name, shape in _SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(theta[o:o + k]).reshape(shape)
        o += k
    return out


def pack(parts):
    return np.concatenate([np.asarray(parts[name]).reshape(-1) for name, _ in _SHAPES])


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = ((u + (((u >> 16) & 1) + 0x7FFF)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def features(centroids, normals, areas, rhs):
    """The 16 per-panel inputs (8 used): centroid relative to the mean centroid
    over the RMS radius R, unit normal, log(area / R^2), rhs / RMS rhs."""
    c = np.asarray(centroids, np.float64)
    n = c.shape[0]
    mc = c.mean(axis=0)
    R = np.sqrt(((c - mc) ** 2).sum(axis=1).mean()) or 1.0
    a = np.asarray(areas, np.float64)
    b = np.asarray(rhs, np.float64)
    rb = np.sqrt((b * b).mean()) or 1.0
    f = np.zeros((n, INPUTS), np.float32)
    f[:, 0:3] = (c - mc) / R
    f[:, 3:6] = np.asarray(normals, np.float64)
    f[:, 6] = np.where(a > 0, np.log(np.where(a > 0, a, 1.0) / (R * R)), 0.0)
    f[:, 7] = b / rb
    return f


def _round(x, on):
    return bf16(x).astype(np.float64) if on else np.asarray(x, np.float64)


def forward(theta, feats, emulate_bf16=True):
    P = {k: np.asarray(v, np.float64) for k, v in unpack(theta).items()}
    r = lambda x: _round(x, emulate_bf16)
    W1, W2, W3 = ((bf16(P[k]).astype(np.float64) if emulate_bf16 else P[k]) for k in ("W1", "W2", "W3"))
    x0 = r(feats)
    h1 = r(np.maximum(x0 @ W1.T + P["b1"], 0.0))
    g = h1.mean(axis=0)
    c2 = P["V2"] @ g + P["b2"]
    h2 = r(np.maximum(h1 @ W2.T + c2, 0.0))
    h3 = r(np.maximum(h2 @ W3.T + P["b3"], 0.0))
    y = h3 @ P["w4"] + P["b4"][0]
    cache = dict(x0=x0, h1=h1, g=g, h2=h2, h3=h3, W2=W2, W3=W3)
    return y, cache


def loss(y, scale, sigma, areas):
    """L = sum A (s (1 + y) - sigma)^2 / sum A sigma^2 and dL/dy."""
    e = scale * (1.0 + y) - sigma
    den = float(np.sum(areas * sigma * sigma)) or 1.0
    return float(np.sum(areas * e * e)) / den, 2.0 * areas * e * scale / den


def backward(theta, cache, dy, emulate_bf16=True):
    P = {k: np.asarray(v, np.float64) for k, v in unpack(theta).items()}
    r = lambda x: _round(x, emulate_bf16)
    x0, h1, g, h2, h3, W2, W3 = (cache[k] for k in ("x0", "h1", "g", "h2", "h3", "W2", "W3"))
    n = x0.shape[0]
    G = {}
    G["w4"] = h3.T @ dy
    G["b4"] = np.array([dy.sum()])
    dz3 = r((h3 > 0) * dy[:, None] * P["w4"][None, :])
    G["W3"] = dz3.T @ h2
    G["b3"] = dz3.sum(axis=0)
    dz2 = r((h2 > 0) * (dz3 @ W3))
    G["W2"] = dz2.T @ h1
    G["b2"] = dz2.sum(axis=0)
    G["V2"] = np.outer(G["b2"], g)
    dg = P["V2"].T @ G["b2"] / n
    dz1 = r((h1 > 0) * (dz2 @ W2 + dg[None, :]))
    G["W1"] = dz1.T @ x0
    G["b1"] = dz1.sum(axis=0)
    return pack(G)


def init(seed=0):
    """He-normal weights, zero biases, small output layer (the network starts
    close to y = 0, i.e. the base guess it corrects)."""
    rng = np.random.default_rng(seed)
    P = {}
    P["W1"] = rng.normal(0, np.sqrt(2.0 / 8), (WIDTH, INPUTS))
    P["W1"][:, 8:] = 0.0
    P["b1"] = np.zeros(WIDTH)
    P["W2"] = rng.normal(0, np.sqrt(2.0 / WIDTH), (WIDTH, WIDTH))
    P["V2"] = rng.normal(0, np.sqrt(1.0 / WIDTH), (WIDTH, WIDTH))
    P["b2"] = np.zeros(WIDTH)
    P["W3"] = rng.normal(0, np.sqrt(2.0 / WIDTH), (WIDTH, WIDTH))
    P["b3"] = np.zeros(WIDTH)
    P["w4"] = rng.normal(0, 1e-3, WIDTH)
    P["b4"] = np.zeros(1)
    return pack(P).astype(np.float32)
