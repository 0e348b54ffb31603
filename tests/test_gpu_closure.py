"""The learned stress closure end to end: samples harvested from states the
plain solver produced, fp64 return-map labels (the yielding samples kept),
training on the GPU with the tensor-core kernels, the closure inside the
substep kernel, and what the trained network gains (or costs) against the
method without it -- the SVD plus return map -- in accuracy and in
particle-substeps per second.

The scene is the snow/sand collision at reduced size: two 40^3 boxes at
2 particles per cell axis (128k particles) on dx = 1/256."""

import time

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, scenes
from squishy_volumes_gb300._abi import SV_TOMBSTONED, SvError

from test_gpu_parity import by_norm

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.snow_sand_2m(box_dims=(40, 40, 40), dx=1.0 / 256)


def _harvested(s, rounds=8, per_round=40000, substeps=20):
    g = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    total = 0
    for k in range(rounds):
        assert g.step(substeps, s.dt, s.gravity) == (0, substeps)
        total = g.closure_harvest(s.dt, per_round, 0.02, seed=k)
    return g, total


@pytest.fixture(scope="module")
def trained():
    s = _scene()
    g, total = _harvested(s)
    loss = g.closure_train(6000, 16384, 3e-3, seed=1)
    yield s, g, total, loss
    g.close()


def test_harvest_and_training(cuda_lib, trained):
    s, g, total, loss = trained
    assert 100_000 < total <= 8 * 40000
    print(f"pool {total}, loss (normalised units) {loss:.3e}")
    assert np.isfinite(loss) and loss < 2e-2
    p = g.closure_params()
    assert p.shape == (g.closure_params().size,) and np.isfinite(p).all()


def test_training_is_what_lets_the_network_take_over(cuda_lib, trained):
    """The same pipeline with zero training steps (He-initialised network):
    its residual check rejects almost every particle the network is asked
    about, so they fall back to the return map; the trained network passes
    it almost everywhere."""
    s, g, _, _ = trained
    ev = g.closure_evaluate(s.dt)
    g0, _ = _harvested(s, rounds=1)
    g0.closure_train(0, 8192, 3e-3, seed=1)
    ev0 = g0.closure_evaluate(s.dt)
    g0.close()
    print(ev0, ev)
    assert ev0["network"] > 0 and ev["network"] > 0
    assert ev0["residual_rejects"] > 0.9 * ev0["network"], ev0
    assert ev["residual_rejects"] < 0.15 * ev["network"], ev


def test_learned_closure_error_and_fallbacks(cuda_lib, trained):
    s, g, _, _ = trained
    ev = g.closure_evaluate(s.dt)
    print(ev)
    assert ev["particles"] == s.io_state.particles.n
    assert ev["fallbacks"] < 0.1 * ev["particles"]
    # fp32 return map: rounding-level
    assert ev["stress_err_plain32"] < 1e-4
    assert ev["stress_err_learned"] < 5e-2
    assert ev["f_err_learned"] < 1e-3


def test_copy_to_another_handle(cuda_lib, trained):
    """A network trained on one handle, handed to another: the same
    evaluation on the same state."""
    s, g, _, _ = trained
    from squishy_volumes_gb300 import IoState

    other = CudaState.from_io_state(IoState(0.0, g.download()), s.consts, s.extras)
    with pytest.raises(SvError):
        other.closure_set_mode(1)
    other.closure_copy_from(g)
    np.testing.assert_array_equal(other.closure_params(), g.closure_params())
    a, b = g.closure_evaluate(s.dt), other.closure_evaluate(s.dt)
    # the sums are fp64 atomics: equal up to their order
    for k in a:
        assert b[k] == pytest.approx(a[k], rel=1e-9, abs=1e-300), (k, a, b)
    other.closure_set_mode(1)
    assert other.step(4, s.dt, s.gravity) == (0, 4)
    other.close()


def test_phase_times(cuda_lib, trained, record_property):
    """The measured per-phase costs of both paths (recorded, not asserted)."""
    s, g, _, _ = trained
    t = g.closure_phase_times(s.dt)
    print(t)
    for k, v in t.items():
        record_property(k, v)
    assert t["particles"] == s.io_state.particles.n
    assert 0 < t["yielding"] <= t["particles"]
    assert t["plain_ms"] > 0 and t["closed_form_ms"] > 0 and t["network_all_ms"] > 0


def test_learned_mode_substeps_stay_close_to_plain(cuda_lib, trained):
    s, g, _, _ = trained
    state = g.download()
    from squishy_volumes_gb300 import IoState

    plain = CudaState.from_io_state(IoState(0.0, state), s.consts, s.extras)
    g.closure_set_mode(1)
    n = 40
    before = g.stats()
    assert g.step(n, s.dt, s.gravity) == (0, n)
    assert plain.step(n, s.dt, s.gravity) == (0, n)
    after = g.stats()
    g.closure_set_mode(0)
    a, b = g.download(), plain.download()
    plain.close()
    learned = after["closure_learned"] - before["closure_learned"]
    fallbacks = after["closure_fallbacks"] - before["closure_fallbacks"]
    assert learned + fallbacks == n * s.io_state.particles.n
    assert fallbacks < 0.1 * learned
    np.testing.assert_array_equal(a.flags & SV_TOMBSTONED, b.flags & SV_TOMBSTONED)
    print(f"after {n} substeps learned vs plain: x {by_norm(a.positions, b.positions, 0)[1]:.2e} "
          f"v {by_norm(a.velocities, b.velocities, 0)[1]:.2e} F "
          f"{by_norm(a.position_gradients, b.position_gradients, 0)[1]:.2e}")
    ok, r = by_norm(a.positions, b.positions, 1e-3)
    assert ok, r
    ok, r = by_norm(a.velocities, b.velocities, 0.2)
    assert ok, r


def test_gain_over_the_return_map(cuda_lib, trained, record_property):
    """Particle-substeps/s of the learned closure against the SVD + return
    map on the same state; recorded, not asserted: on GB300 the network pass
    costs more than the fp32 Jacobi SVD and closed-form return maps it
    replaces (see the design notes)."""
    import torch

    s, g, _, _ = trained
    n, rates = 60, {}
    for mode in (0, 1, 0, 1):
        g.closure_set_mode(mode)
        g.step(8, s.dt, s.gravity)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        assert g.step(n, s.dt, s.gravity) == (0, n)
        torch.cuda.synchronize()
        rates[mode] = s.io_state.particles.n * n / (time.perf_counter() - t0)
    g.closure_set_mode(0)
    record_property("plain_particle_substeps_per_s", rates[0])
    record_property("learned_particle_substeps_per_s", rates[1])
    print(f"plain {rates[0]:.3e}  learned {rates[1]:.3e}  ratio {rates[1] / rates[0]:.3f}")
    assert rates[0] > 0 and rates[1] > 0


def test_mode_requires_training(cuda_lib):
    s = _scene()
    g = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    with pytest.raises(SvError):
        g.closure_set_mode(1)
    with pytest.raises(SvError):
        g.closure_train(10)  # empty pool
    g.close()


def test_pool_counts(cuda_lib, trained):
    s, g, total, _ = trained
    p = g.closure_pool()
    assert p["pairs"] == total
    assert 128 <= p["yielding_pairs"] <= total


def test_material_ranges_cover_the_hull(cuda_lib):
    """Labels drawn over material ranges: the pool's lambda / mu feature then
    spans the ranges' ends whichever scenes the samples came from."""
    s = _scene()
    g, _ = _harvested(s, rounds=2)
    with pytest.raises(SvError):
        g.closure_set_material_ranges((0.3, 0.2), (25.0, 40.0))
    with pytest.raises(SvError):
        g.closure_set_material_ranges((0.2, 0.4), (25.0, 95.0))
    g.closure_set_material_ranges((0.18, 0.42), (23.0, 42.0))
    g.closure_train(0, 8192, 3e-3, seed=1)
    _, _, hull = g.closure_training_pool(0, 1)
    lo, hi = 2 * 0.18 / (1 - 0.36), 2 * 0.42 / (1 - 0.84)
    assert hull["lo"][5] <= lo * 1.01 and hull["hi"][5] >= hi * 0.99, hull
    # alpha of 23 and 42 degrees (feature 8, sand)
    a = lambda d: np.sqrt(2 / 3) * 2 * np.sin(np.radians(d)) / (3 - np.sin(np.radians(d)))
    assert hull["hi"][8] >= a(42.0) * 0.99, hull
    g.close()


def test_harvest_from_another_handle(cuda_lib):
    """One pool gathers another handle's states: the samples carry their
    materials, so the labels do not depend on the pool handle's table."""
    s = _scene()
    pool = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    other = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    for k in range(4):
        assert other.step(20, s.dt, s.gravity) == (0, 20)
        total = pool.closure_harvest_from(other, s.dt, 20000, 0.02, seed=k)
    assert 20000 < total <= 80000
    pool.closure_train(0, 8192, 3e-3, seed=1)
    X, Y, hull = pool.closure_training_pool()
    assert pool.closure_pool()["yielding_pairs"] == X.shape[0] > 0
    # snow and sand both in the pool (features 3 and 4 are the one-hot kinds)
    raw = X[:, 3] / hull["xs"][3] + hull["xm"][3]
    assert (raw > 0.5).any() and (raw < 0.5).any()
    other.close()
    pool.close()
