"""CPU oracle of the learned form's network: forward pass, loss and gradients
in FP64 numpy, used by the tests to check the GPU training kernels
(gcurval_gb300/csrc/gcv_mlp_train.cu) and the tensor-core inference.

Test infrastructure only.  The network has no counterpart in the reference;
its definition is the library's (include/gcurval_gb300_learned.h):
16 -> 128 -> 128 -> 128 (GELU, tanh form) -> 32; loss = cross-entropy of the
13 depth logits + soft cross-entropy of the 4 quarter logits against the leaf
shares + half the squared error of the 8 parameters, averaged over rows.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 16, 128, 32
SHAPES = [("W1", (IN, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
          ("W4", (H, OUT)), ("b4", (OUT,))]
N_PARAM = sum(int(np.prod(s)) for _, s in SHAPES)
C = np.sqrt(2.0 / np.pi)
A = 0.044715


def unpack(w):
    w = np.asarray(w, np.float64)
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = w[o:o + n].reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in SHAPES])


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C * (x + A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C * (x + A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C * (1.0 + 3.0 * A * x * x)


def forward(w, X):
    p = unpack(w)
    acts = []
    h = np.asarray(X, np.float64)
    for l in (1, 2, 3):
        z = h @ p[f"W{l}"] + p[f"b{l}"]
        acts.append((h, z))
        h = gelu(z)
    out = h @ p["W4"] + p["b4"]
    return out, acts, h


def _softmax(z):
    z = z - z.max(axis=1, keepdims=True)
    e = np.exp(z)
    return e / e.sum(axis=1, keepdims=True)


def loss_and_grad(w, X, depth, share, tg):
    """(mean loss parts [depth, split, t], gradient packed like w)."""
    p = unpack(w)
    out, acts, h3 = forward(w, X)
    n = X.shape[0]
    depth = np.asarray(depth, np.int64)
    share = np.asarray(share, np.float64)
    tg = np.asarray(tg, np.float64)
    pd = _softmax(out[:, :13])
    ps = _softmax(out[:, 13:17])
    l0 = -np.log(pd[np.arange(n), depth]).mean()
    l1 = -(share * np.log(ps)).sum(axis=1).mean()
    e = out[:, 17:25] - tg
    l2 = 0.5 * (e * e).sum(axis=1).mean()
    d_out = np.zeros_like(out)
    onehot = np.zeros_like(pd)
    onehot[np.arange(n), depth] = 1.0
    d_out[:, :13] = (pd - onehot) / n
    d_out[:, 13:17] = (ps - share) / n
    d_out[:, 17:25] = e / n
    g = {"W4": h3.T @ d_out, "b4": d_out.sum(axis=0)}
    dh = d_out @ p["W4"].T
    for l in (3, 2, 1):
        h_in, z = acts[l - 1]
        dz = dh * gelu_grad(z)
        g[f"W{l}"] = h_in.T @ dz
        g[f"b{l}"] = dz.sum(axis=0)
        dh = dz @ p[f"W{l}"].T
    return np.array([l0, l1, l2]), pack(g)


def he_init(seed=0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("W"):
            d[name] = rng.normal(0.0, np.sqrt(2.0 / shp[0]), shp)
        else:
            d[name] = rng.normal(0.0, 0.1, shp)
    return pack(d)
