"""The CPU checker of the learned closure's network, pinned on its own:
bf16 rounding known answers and the backward pass against central finite
differences of the float64 network."""

import numpy as np

from oracle import closure as oc


def test_bf16_rounding_known_answers():
    # bf16 keeps 7 explicit mantissa bits: spacing 2^-7 in [1, 2)
    vals = np.array([1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e38],
                    np.float64)
    exp = np.array([1.0, 1.0 + 2 ** -7, 1.0, 1.0 + 2 ** -6, 1.0, -2.5, 0.0])
    got = oc.bf16(vals)
    np.testing.assert_array_equal(got[:7], exp)  # ties go to even
    assert abs(got[7] - vals[7]) / vals[7] <= 2 ** -8  # within half a bf16 ulp


def test_param_count_and_layout():
    # four hidden layers of width 64 and an 8-output head
    assert oc.N_PARAMS == 64 * 16 + 64 + 3 * (64 * 64 + 64) + 8 * 64 + 8
    p = np.arange(oc.N_PARAMS, dtype=np.float32)
    d = oc.unpack(p)
    assert d["W1"][1, 0] == 16 and d["b1"][0] == 1024 and d["W4"].shape == (64, 64) and d["W5"].shape == (8, 64)
    np.testing.assert_array_equal(oc.pack(d), p)


def test_silu_and_its_derivative():
    z = np.linspace(-8, 8, 41)
    np.testing.assert_allclose(oc.silu(z), z / (1 + np.exp(-z)), rtol=1e-14)
    eps = 1e-6
    np.testing.assert_allclose(oc.silu_grad(z), (oc.silu(z + eps) - oc.silu(z - eps)) / (2 * eps), rtol=1e-7, atol=1e-9)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(2)
    n = 9
    params = oc.init_params(7).astype(np.float64)
    params += rng.normal(0, 0.05, params.shape)  # non-zero biases too
    x = rng.normal(0, 1.0, (n, oc.NIN))
    t = rng.normal(0, 1.0, (n, oc.NOUT))
    w = rng.uniform(0.5, 1.5, n)
    _, loss, g = oc.loss_and_grad(params, x, t, w, rounding=False)
    eps = 1e-6
    idx = rng.choice(oc.N_PARAMS, 120, replace=False)
    num = np.empty(len(idx))
    for j, i in enumerate(idx):
        pp, pm = params.copy(), params.copy()
        pp[i] += eps
        pm[i] -= eps
        num[j] = (oc.loss_and_grad(pp, x, t, w, rounding=False)[1] - oc.loss_and_grad(pm, x, t, w, rounding=False)[1]) / (2 * eps)
    np.testing.assert_allclose(g[idx], num, rtol=1e-5, atol=1e-8)
    assert loss > 0
