"""Host side of the learned stress closure: thin wrappers over the C ABI.

The network (x 16 -> four hidden layers of width 64 with SiLU, bf16
tensor-core operands with fp32 accumulation -> an fp32 head of 8 outputs)
runs only in the CUDA library; these functions move host arrays in and out.
"""

from __future__ import annotations

import ctypes as ct

import numpy as np

from ._abi import check, f32p, load, ptr

NIN, NH, NOUT, N_USED_OUT = 16, 64, 8, 6


def param_count() -> int:
    return int(load().sv_mlp_param_count())


def mlp_forward(params, x) -> np.ndarray:
    """y[n, 8] = network(x[n, 16]) on the GPU (input 15 is read as 0)."""
    params = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, NIN)
    y = np.zeros((x.shape[0], NOUT), np.float32)
    check(load().sv_mlp_forward(ptr(params, f32p), ptr(x, f32p), x.shape[0], ptr(y, f32p)))
    return y


def mlp_grad(params, x, t, w):
    """(y, loss, grad) of sum_r w_r sum_{o<6} (y_ro - t_ro)^2 / n on the GPU."""
    params = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, NIN)
    n = x.shape[0]
    t = np.ascontiguousarray(t, np.float32).reshape(n, NOUT)
    w = np.ascontiguousarray(w, np.float32).reshape(n)
    y = np.zeros((n, NOUT), np.float32)
    g = np.zeros(param_count(), np.float32)
    loss = ct.c_float(0.0)
    check(load().sv_mlp_grad(ptr(params, f32p), ptr(x, f32p), ptr(t, f32p), ptr(w, f32p), n, ptr(y, f32p),
                             ptr(g, f32p), ct.byref(loss)))
    return y, float(loss.value), g
