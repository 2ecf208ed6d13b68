"""CPU oracle of the learned-MTS network (test infrastructure only).

The per-atom MLP of the learned multiple-time-step form has no counterpart in
the reference, so this is a restatement of the standard published algorithm
(dense layers, SiLU, mean-squared error, reverse-mode backpropagation) in
numpy FP64.  With ``bf16=True`` it rounds at the same points as the CUDA
kernels: inputs, weights, hidden activations and the activation gradients are
rounded to bfloat16 (round to nearest even), and everything else is FP64, so
the CUDA FP32 accumulation can be checked against it.  With ``bf16=False`` it
is the exact FP64 gradient of the FP64 loss (checked by finite differences).

Parameter vector layout (FP32 in the library):
    W1[51][128] b1[128] W2[128][128] b2[128] W3[128][3] b3[3]

Only tests may import this module; the product path never calls it.
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 51, 128, 3
SHAPES = (("W1", (NIN, NH)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NH, NOUT)), ("b3", (NOUT,)))
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(a) -> np.ndarray:
    """Round to bfloat16 (nearest even) via float32, returned as float64."""
    f = np.asarray(a, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, np.float64)
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SHAPES])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(x, params, bf16_points: bool = True):
    """Network output y[nb][3] and the intermediates of the forward pass."""
    r = bf16 if bf16_points else (lambda a: np.asarray(a, np.float64))
    P = unpack(params)
    xb = r(x)
    W1, W2, W3 = r(P["W1"]), r(P["W2"]), r(P["W3"])
    z1 = xb @ W1 + P["b1"]
    h1 = r(silu(z1))
    z2 = h1 @ W2 + P["b2"]
    h2 = r(silu(z2))
    y = h2 @ W3 + P["b3"]
    return y, dict(x=xb, W1=W1, W2=W2, W3=W3, z1=z1, h1=h1, z2=z2, h2=h2)


def loss_and_grad(x, target, params, bf16_points: bool = True):
    """Mean-squared error over nb*3 outputs and its gradient (packed)."""
    r = bf16 if bf16_points else (lambda a: np.asarray(a, np.float64))
    y, c = forward(x, params, bf16_points)
    t = np.asarray(target, np.float64)
    cnt = y.size
    d = y - t
    loss = float((d * d).sum() / cnt)
    dy = r(2.0 * d / cnt)
    g = {}
    g["W3"] = c["h2"].T @ dy
    g["b3"] = dy.sum(0)
    dz2 = r((dy @ c["W3"].T) * dsilu(c["z2"]))
    g["W2"] = c["h1"].T @ dz2
    g["b2"] = dz2.sum(0)
    dz1 = r((dz2 @ c["W2"].T) * dsilu(c["z1"]))
    g["W1"] = c["x"].T @ dz1
    g["b1"] = dz1.sum(0)
    return loss, pack(g), y


def initial_params(seed: int = 7, out_gain: float = 0.1) -> np.ndarray:
    """Glorot-uniform weights and zero biases (a test starting point)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("b"):
            d[name] = np.zeros(shape)
        else:
            a = np.sqrt(6.0 / (shape[0] + shape[1])) * (out_gain if name == "W3" else 1.0)
            d[name] = rng.uniform(-a, a, shape)
    return pack(d)
