"""CPU checker for the learned stress closure (test infrastructure only).

The closure is an addition, not part of the reference, so there is nothing of
the reference to restate here.  This module evaluates the same small MLP as
the tensor-core kernels in squishy_volumes_gb300/csrc/sv_mlp.cu -- forward
pass, loss and backward pass -- in numpy float64, rounding to bf16 at exactly
the points where the kernels hand a value to the tensor core (inputs,
weights, hidden activations, and the gradients that enter the backward
products).  With rounding switched off it is the plain float64 network, whose
backward pass the tests pin by finite differences.

Parameter vector layout (fp32 master copy, row-major, out x in):
W1 [NH, NIN], b1 [NH], W2 [NH, NH], b2 [NH], W3 [NOUT, NH], b3 [NOUT].
Loss: sum over rows r and outputs o < N_USED_OUT of w_r (y_ro - t_ro)^2 / n.
"""

from __future__ import annotations

import numpy as np

NIN, NH, NOUT, N_USED_OUT = 16, 32, 16, 6
SHAPES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NOUT, NH)), ("b3", (NOUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(params):
    out, o = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = np.asarray(params[o:o + size], np.float64).reshape(shape)
        o += size
    return out


def pack(d, dtype=np.float32):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SHAPES]).astype(dtype)


def bf16(a):
    """Round to the nearest bf16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def init_params(seed: int, scale: float = 1.0):
    """He-style initial weights, zero biases (the trainer's initialisation)."""
    rng = np.random.default_rng(seed)
    d = {
        "W1": rng.normal(0.0, scale * np.sqrt(2.0 / NIN), (NH, NIN)),
        "b1": np.zeros(NH),
        "W2": rng.normal(0.0, scale * np.sqrt(2.0 / NH), (NH, NH)),
        "b2": np.zeros(NH),
        "W3": rng.normal(0.0, scale * np.sqrt(1.0 / NH), (NOUT, NH)),
        "b3": np.zeros(NOUT),
    }
    return pack(d)


def forward(params, x, rounding=True):
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    xb = r(x)
    z1 = xb @ r(p["W1"]).T + p["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = r(h1) @ r(p["W2"]).T + p["b2"]
    h2 = np.maximum(z2, 0.0)
    y = r(h2) @ r(p["W3"]).T + p["b3"]
    return y, (xb, z1, h1, z2, h2)


def loss_and_grad(params, x, t, w, rounding=True):
    """(y, loss, grad) of the weighted squared error over the first
    N_USED_OUT outputs."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    n = x.shape[0]
    y, (xb, z1, h1, z2, h2) = forward(params, x, rounding)
    w = np.asarray(w, np.float64)[:, None]
    d = np.zeros_like(y)
    d[:, :N_USED_OUT] = y[:, :N_USED_OUT] - np.asarray(t, np.float64)[:, :N_USED_OUT]
    loss = float((w * d * d).sum() / n)
    dy = 2.0 * w * d / n
    # the kernels round dY to bf16 before both backward products
    dyb = r(dy)
    g = {"b3": dy.sum(0), "W3": dyb.T @ r(h2)}
    dh2 = dyb @ r(p["W3"])
    dz2 = dh2 * (z2 > 0)
    dz2b = r(dz2)
    g["b2"] = dz2.sum(0)
    g["W2"] = dz2b.T @ r(h1)
    dh1 = dz2b @ r(p["W2"])
    dz1 = dh1 * (z1 > 0)
    g["b1"] = dz1.sum(0)
    g["W1"] = r(dz1).T @ xb
    return y, loss, pack(g, np.float64)
