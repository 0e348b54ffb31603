"""The tensor-core MLP kernels of the learned closure (tcgen05 MMAs with
TMEM accumulators) against the CPU checker, which rounds to bf16 where the
kernels feed the tensor core.  Remaining differences come from fp32
accumulation order, from the kernels' SiLU (fast exponential and reciprocal)
and from rare bf16 re-rounding of an activation that sits on a rounding
boundary, hence the norm tolerances.  Network: 16 -> 4 x 64 SiLU -> 8."""

import numpy as np
import pytest

from oracle import closure as oc
from squishy_volumes_gb300 import closure

pytestmark = pytest.mark.gpu


def _params(seed):
    rng = np.random.default_rng(seed)
    p = oc.init_params(seed).astype(np.float64)
    p += rng.normal(0, 0.05, p.shape)
    return p.astype(np.float32)


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_param_count(cuda_lib):
    assert closure.param_count() == oc.N_PARAMS


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 40000])
def test_forward_matches_cpu(cuda_lib, n):
    params = _params(1)
    x = np.random.default_rng(n).normal(0, 1.0, (n, oc.NIN)).astype(np.float32)
    y = closure.mlp_forward(params, x)
    ref, _ = oc.forward(params, x, rounding=True)
    assert _rel(y, ref) < 3e-4
    # input 15 is reserved: the kernels read it as zero
    x2 = x.copy()
    x2[:, oc.NIN - 1] = 123.0
    np.testing.assert_array_equal(closure.mlp_forward(params, x2), y)
    # without the bf16 emulation the difference is bf16-sized, not larger
    ref64, _ = oc.forward(params, x, rounding=False)
    assert _rel(y, ref64) < 3e-2


@pytest.mark.parametrize("n", [5, 128, 3000, 50000])
def test_gradient_matches_cpu(cuda_lib, n):
    """50k rows are 391 tiles over one CTA per SM: CTAs accumulate the
    weight gradients of several tiles in TMEM."""
    rng = np.random.default_rng(100 + n)
    params = _params(2)
    x = rng.normal(0, 1.0, (n, oc.NIN)).astype(np.float32)
    t = rng.normal(0, 1.0, (n, oc.NOUT)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, n).astype(np.float32)
    y, loss, g = closure.mlp_grad(params, x, t, w)
    yr, lr, gr = oc.loss_and_grad(params, x, t, w, rounding=True)
    assert _rel(y, yr) < 3e-4
    assert abs(loss - lr) <= 3e-4 * lr
    assert _rel(g, gr) < 3e-3
    o = 0
    for name, shape in oc.SHAPES:
        size = int(np.prod(shape))
        assert _rel(g[o:o + size], gr[o:o + size]) < 1e-2, name
        o += size


def test_empty_batch(cuda_lib):
    params = _params(3)
    x = np.zeros((0, oc.NIN), np.float32)
    assert closure.mlp_forward(params, x).shape == (0, oc.NOUT)
    y, loss, g = closure.mlp_grad(params, x, np.zeros((0, oc.NOUT)), np.zeros(0))
    assert loss == 0.0 and not g.any()


def test_unused_outputs_get_no_gradient(cuda_lib):
    """Outputs 6 and 7 are outside the loss: the head rows that produce them
    get exactly zero gradient, as does W1's reserved input column."""
    rng = np.random.default_rng(7)
    n = 700
    params = _params(4)
    x = rng.normal(0, 1.0, (n, oc.NIN)).astype(np.float32)
    t = rng.normal(0, 1.0, (n, oc.NOUT)).astype(np.float32)
    _, _, g = closure.mlp_grad(params, x, t, np.ones(n, np.float32))
    d = oc.unpack(g)
    assert not d["W5"][oc.N_USED_OUT:].any() and not d["b5"][oc.N_USED_OUT:].any()
    assert not d["W1"][:, oc.NIN - 1].any()
    assert d["W5"][:oc.N_USED_OUT].any()
