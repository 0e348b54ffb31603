"""CPU checker for the learned stress closure (test infrastructure only).

The closure is an addition, not part of the reference, so there is nothing of
the reference to restate here.  This module evaluates the same network as
the tensor-core kernels in squishy_volumes_gb300/csrc/sv_mlp.cu -- forward
pass, loss and backward pass -- in numpy float64, rounding to bf16 at exactly
the points where the kernels hand a value to the tensor core (inputs,
weights, hidden activations, and the gradients that enter the backward
products).  With rounding switched off it is the plain float64 network, whose
backward pass the tests pin by finite differences.

Network: x (16, input 15 reserved and zero) -> four hidden layers of width 64
with SiLU, silu(z) = z / (1 + exp(-z)) -> an fp32 head of 8 outputs (the
first 6 used).  The hidden layers run on the tensor cores (bf16 operands,
fp32 accumulation); the head reads the last hidden layer in fp32.

Parameter vector layout (fp32 master copy, row-major, out x in):
W1 [64, 16], b1 [64], W2 [64, 64], b2, W3 [64, 64], b3, W4 [64, 64], b4,
W5 [8, 64], b5 [8].
Loss: sum over rows r and outputs o < N_USED_OUT of w_r (y_ro - t_ro)^2 / n.

The kernels take each bias gradient out of the weight-gradient product of
its layer (a constant row of ones next to the layer's input), so a bias
gradient sums the bf16-rounded pre-activation gradients, as here.
"""

from __future__ import annotations

import numpy as np

NIN, NH, NOUT, N_USED_OUT = 16, 64, 8, 6
N_HIDDEN = 4
SHAPES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NH, NH)), ("b3", (NH,)),
          ("W4", (NH, NH)), ("b4", (NH,)), ("W5", (NOUT, NH)), ("b5", (NOUT,))]
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


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def silu_grad(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def init_params(seed: int, scale: float = 1.0):
    """He-style initial weights, zero biases (the trainer's initialisation)."""
    rng = np.random.default_rng(seed)
    d = {"W1": rng.normal(0.0, scale * np.sqrt(2.0 / NIN), (NH, NIN)), "b1": np.zeros(NH)}
    for k in (2, 3, 4):
        d[f"W{k}"] = rng.normal(0.0, scale * np.sqrt(2.0 / NH), (NH, NH))
        d[f"b{k}"] = np.zeros(NH)
    d["W5"] = rng.normal(0.0, scale * np.sqrt(1.0 / NH), (NOUT, NH))
    d["b5"] = np.zeros(NOUT)
    return pack(d)


def forward(params, x, rounding=True):
    """y [n, 8] and the intermediates (xb, z1..z4, h1..h4)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    x = np.array(x, np.float64)
    x[:, NIN - 1] = 0.0  # input 15 is reserved: the kernels read it as zero
    xb = r(x)
    zs, hs = [], []
    a = xb
    for k in range(1, N_HIDDEN + 1):
        z = a @ r(p[f"W{k}"]).T + p[f"b{k}"]
        h = silu(z)
        zs.append(z)
        hs.append(h)
        a = r(h)
    y = hs[-1] @ p["W5"].T + p["b5"]  # fp32 head: the last hidden layer is not rounded
    return y, (xb, zs, hs)


def loss_and_grad(params, x, t, w, rounding=True):
    """(y, loss, grad) of the weighted squared error over the first
    N_USED_OUT outputs."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    n = x.shape[0]
    y, (xb, zs, hs) = forward(params, x, rounding)
    w = np.asarray(w, np.float64)[:, None]
    d = np.zeros_like(y)
    d[:, :N_USED_OUT] = y[:, :N_USED_OUT] - np.asarray(t, np.float64)[:, :N_USED_OUT]
    loss = float((w * d * d).sum() / n)
    dy = 2.0 * w * d / n
    g = {}
    # head: weight and bias gradients from the tensor core (bf16 dY and h4),
    # the input gradient in fp32
    dyb = r(dy)
    g["W5"] = dyb.T @ r(hs[3])
    g["b5"] = dyb.sum(0)
    dh = dy @ p["W5"]
    inputs = [xb] + [r(h) for h in hs[:3]]
    for k in range(N_HIDDEN, 0, -1):
        dz = dh * silu_grad(zs[k - 1])
        dzb = r(dz)
        g[f"W{k}"] = dzb.T @ inputs[k - 1]
        g[f"b{k}"] = dzb.sum(0)
        if k > 1:
            dh = dzb @ r(p[f"W{k}"])
    return y, loss, pack(g, np.float64)
