"""Learned insertion proposal, restated in float64 NumPy (test infrastructure).

No counterpart exists in the reference: the proposal enters through the
ChangesFn log proposal ratio of the exchange move (src/kups/mcmc/moves.py:92-98,
summed into ln acc at src/kups/core/propagator.py:330-334), where the
reference's uniform insertion contributes zero (moves.py:799-801).

The network: features (sin, cos)(2 pi m_j . f) of the fractional position,
three softplus layers of width 256, linear output g.  ``emulate=True`` rounds
every tensor-core operand to bfloat16 at the points the CUDA path does
(features, the weight copies, the stored activations h1 and h2, and the
upstream gradients of the backward GEMMs), so the CUDA path can be compared
tightly; ``emulate=False`` is plain float64 and is what the finite-difference
check of the hand-derived backward pass runs on.

Grid density: node values d_v = exp(g_v - max g) + floor * mean, cell mass =
mean of the 8 corners, q_f(f) = P_c G^3 8 tri(t) / sum(corners).
"""

from __future__ import annotations

import numpy as np

N_FREQ, N_IN, N_HID = 32, 64, 256
OFFSETS = {"W1": (0, (N_HID, N_IN)), "b1": (16384, (N_HID,)), "W2": (16640, (N_HID, N_HID)),
           "b2": (82176, (N_HID,)), "W3": (82432, (N_HID, N_HID)), "b3": (147968, (N_HID,)),
           "w4": (148224, (N_HID,)), "b4": (148480, (1,))}
N_PARAMS = 148481


def unflatten(flat):
    flat = np.asarray(flat, np.float64)
    return {k: flat[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFFSETS.items()}


def flatten(p):
    out = np.zeros(N_PARAMS)
    for k, (o, s) in OFFSETS.items():
        out[o:o + int(np.prod(s))] = np.asarray(p[k]).reshape(-1)
    return out


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def softplus(z):
    return np.where(z > 20, z, np.log1p(np.exp(np.minimum(z, 20))))


def features(x, freq):
    t = np.asarray(x, np.float64) @ np.asarray(freq, np.float64).T  # [n, 32]
    t = t - np.rint(t)
    f = np.empty((len(t), N_IN))
    f[:, 0::2] = np.sin(2 * np.pi * t)
    f[:, 1::2] = np.cos(2 * np.pi * t)
    return f


def forward(p, x, freq, emulate=True):
    """Activations and g for points x [n, 3]."""
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    F = r(features(x, freq))
    h1 = softplus(F @ r(p["W1"]).T + p["b1"])
    h2 = softplus(r(h1) @ r(p["W2"]).T + p["b2"])
    h3 = softplus(r(h2) @ r(p["W3"]).T + p["b3"])
    g = h3 @ p["w4"] + p["b4"][0]
    return dict(F=F, h1=h1, h2=h2, h3=h3, g=g)


def loss_and_grad(p, x, label, freq, emulate=True):
    """Noise-contrastive loss L = mean(y softplus(-g) + (1 - y) softplus(g)) and dL/dparam."""
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    a = forward(p, x, freq, emulate)
    y = np.asarray(label, np.float64)
    n = len(y)
    g = a["g"]
    loss = float(np.mean(np.where(y > 0.5, softplus(-g), softplus(g))))
    dg = (1 / (1 + np.exp(-g)) - y) / n
    gate = lambda h: -np.expm1(-h)  # softplus'(z) written through h = softplus(z)
    dz3 = dg[:, None] * p["w4"][None, :] * gate(a["h3"])
    grads = {"w4": dg @ a["h3"], "b4": np.array([dg.sum()])}
    grads["W3"] = r(dz3).T @ r(a["h2"])
    grads["b3"] = dz3.sum(0)
    dz2 = (r(dz3) @ r(p["W3"])) * gate(a["h2"])
    grads["W2"] = r(dz2).T @ r(a["h1"])
    grads["b2"] = dz2.sum(0)
    dz1 = (r(dz2) @ r(p["W2"])) * gate(a["h1"])
    grads["W1"] = r(dz1).T @ a["F"]
    grads["b1"] = dz1.sum(0)
    return loss, grads


def adam(param, grad, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) on flat arrays; returns (param, m, v)."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1**t)
    vh = v / (1 - beta2**t)
    return param - lr * mh / (np.sqrt(vh) + eps), m, v


def grid_nodes(grid):
    i = np.arange(grid ** 3)
    return np.stack([i // grid**2, (i // grid) % grid, i % grid], 1) / grid


def grid_density(g_nodes, floor_frac, temper=1.0):
    """Node values d from g at the nodes (flat, (i G + j) G + k order)."""
    e = np.exp(temper * (np.asarray(g_nodes, np.float64) - np.max(g_nodes)))
    return e + floor_frac * e.mean()


def cell_masses(node, grid):
    d = np.asarray(node, np.float64).reshape(grid, grid, grid)
    s = np.zeros_like(d)
    for b in range(8):
        s += np.roll(d, (-(b >> 2 & 1), -(b >> 1 & 1), -(b & 1)), (0, 1, 2))
    return (s / 8).reshape(-1)


def cdf_from_node(node, grid):
    return np.concatenate([[0.0], np.cumsum(cell_masses(node, grid))])


def log_q(node, cdf, grid, f):
    """ln q_f (density in fractional measure) at points f [n, 3]."""
    f = np.asarray(f, np.float64)
    f = f - np.floor(f)
    s = f * grid
    c = np.clip(np.floor(s).astype(np.int64), 0, grid - 1)
    t = np.clip(s - c, 0, 1)
    d = np.asarray(node, np.float64).reshape(grid, grid, grid)
    tri = np.zeros(len(f))
    tot = np.zeros(len(f))
    for b in range(8):
        bi = np.array([b >> 2 & 1, b >> 1 & 1, b & 1])
        idx = (c + bi) % grid
        val = d[idx[:, 0], idx[:, 1], idx[:, 2]]
        w = np.prod(np.where(bi == 1, t, 1 - t), 1)
        tri += val * w
        tot += val
    cell = (c[:, 0] * grid + c[:, 1]) * grid + c[:, 2]
    pc = (cdf[cell + 1] - cdf[cell]) / cdf[-1]
    return np.log(pc) + 3 * np.log(grid) + np.log(8 * tri / tot)
