"""Adaptive time steps (the reference's limit_time_step.rs and
AdaptiveTimeStepState) through the C ABI against the fp32 oracle: the same
number of substeps to the target time, the same time steps per phase, the
same limits, and the same state within the whole-substep tolerances."""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, FrameInput, Harness, IoState, RunParameters, scenes
from squishy_volumes_gb300._abi import SV_TOMBSTONED, SvError

from test_gpu_parity import compare_states

pytestmark = pytest.mark.gpu

TOL = {"positions": 1e-5, "velocities": 1e-3, "position_gradients": 1e-4, "elastic_energies": 1e-2}


def _limits_close(gpu_lim, ref_lim, rel=1e-4):
    keys = ("dt_force", "dt_scatter", "dt_advance", "velocity", "deformation", "sound", "isolated", "allowed")
    for k, r in zip(keys, ref_lim):
        g = gpu_lim[k]
        assert abs(g - r) <= rel * abs(r), (k, g, r)


@pytest.mark.parametrize("form", [0, 1])
def test_adaptive_run_matches_oracle(cuda_lib, oracle_mod, form):
    s = scenes.small_mixed()
    target, max_dt = 0.02, 1e-2
    gpu = CudaState.from_io_state(s.io_state, s.consts, Extras(position_form=form))
    status, done, t = gpu.step_adaptive(target, max_dt, s.gravity, time=0.0)
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=False)
    rc, n_ref, t_ref, lim_ref = ref.step_adaptive(0.0, target, max_dt, s.gravity)
    assert (status, rc) == (0, 0)
    assert done == n_ref and done > 3
    assert abs(t - t_ref) <= 1e-5 * t_ref
    _limits_close(gpu.time_step_limits(), lim_ref)
    out, exp = gpu.download(), ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=s.consts.grid_node_size)
    gpu.close()


def test_limit_history_persists_across_calls(cuda_lib, oracle_mod):
    """Two calls (0 -> 0.01 -> 0.02) against the oracle doing the same: the
    prior limits carry over, as in the reference's state."""
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts)
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=False)
    t, tr = 0.0, 0.0
    for target in (0.01, 0.02):
        _, done, t = gpu.step_adaptive(target, 1e-2, s.gravity, time=t)
        _, n_ref, tr, lim_ref = ref.step_adaptive(tr, target, 1e-2, s.gravity)
        assert done == n_ref
        assert abs(t - tr) <= 1e-5 * tr
        _limits_close(gpu.time_step_limits(), lim_ref)
    gpu.close()


def test_velocity_limit_governs_fast_particles(cuda_lib, oracle_mod):
    """Particles at 40 m/s: 0.5 dx / |v| is the smallest limit."""
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.velocities[:] = np.array([40.0, 0.0, 0.0], np.float32)
    p.velocity_gradients[:] = 0
    gpu = CudaState.from_io_state(IoState(0.0, p), s.consts)
    ref = oracle_mod.OracleState(p, s.consts, None, fp64=False)
    _, done, t = gpu.step_adaptive(3e-3, 1e-2, (0, 0, 0), time=0.0)
    _, n_ref, tr, lim_ref = ref.step_adaptive(0.0, 3e-3, 1e-2, (0, 0, 0))
    lim = gpu.time_step_limits()
    assert done == n_ref
    assert lim["velocity"] < min(lim["sound"], lim["isolated"], lim["deformation"])
    _limits_close(lim, lim_ref)
    # The first substep's advance takes the velocity limit's step, below the
    # speculative one (no velocity limit among the priors yet), so its pass
    # is redone; the state still matches the oracle's.
    out, exp = gpu.download(), ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=s.consts.grid_node_size)
    gpu.close()


def test_target_already_reached_runs_nothing(cuda_lib):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts)
    before = gpu.download()
    assert gpu.step_adaptive(0.5, 1e-2, s.gravity, time=0.5) == (0, 0, 0.5)
    after = gpu.download()
    np.testing.assert_array_equal(before.positions, after.positions)
    with pytest.raises(SvError):
        gpu.step_adaptive(1.0, 0.0, s.gravity, time=0.0)  # no positive step
    gpu.close()


def test_produce_next_state_adaptive_and_back_to_fixed(cuda_lib, oracle_mod):
    """produce_next_state with adaptive_time_steps, then fixed steps on the
    same handle: the fused path picks up the state the adaptive path left."""
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts)
    io, err = gpu.produce_next_state(Harness(), FrameInput(s.consts, s.gravity),
                                     RunParameters(target_time=0.01, max_time_step=1e-2, adaptive_time_steps=True))
    assert err is None and gpu.time >= 0.01
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=False)
    _, _, tr, _ = ref.step_adaptive(0.0, 0.01, 1e-2, s.gravity)
    assert abs(gpu.time - tr) <= 1e-5 * tr
    assert gpu.step(5, 1e-3, s.gravity) == (0, 5)
    assert ref.step(5, 1e-3, s.gravity) == 0
    out, exp = gpu.download(), ref.download()
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=s.consts.grid_node_size)
    gpu.close()


@pytest.mark.parametrize("sort_interval", [8, 1])
def test_stale_binning_recovers_like_the_reference(cuda_lib, oracle_mod, sort_interval):
    """Adaptive substeps bin every sort_interval substeps; particles crossing
    half a cell per substep leave their claimed blocks in between, the
    substep is redone from its start (limit history included) after a fresh
    binning, and the run still matches the oracle, which bins every
    substep."""
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    dx = s.consts.grid_node_size
    p.velocities[:] = np.array([30.0, -24.0, 18.0], np.float32)  # the velocity limit: 0.5 cells per substep
    p.velocity_gradients[:] = 0
    target, max_dt = 0.015, 1e-2
    gpu = CudaState.from_io_state(IoState(0.0, p), s.consts, Extras(sort_interval=sort_interval))
    status, done, t = gpu.step_adaptive(target, max_dt, (0, 0, 0), time=0.0)
    ref = oracle_mod.OracleState(p, s.consts, None, fp64=False)
    rc, n_ref, t_ref, lim_ref = ref.step_adaptive(0.0, target, max_dt, (0, 0, 0))
    assert (status, rc) == (0, 0)
    assert done == n_ref and done > 8
    assert abs(t - t_ref) <= 1e-5 * t_ref
    # at 42 m/s of near-rigid motion C is a small difference of large terms:
    # particles outside a stale tile take the unfactorised global gather,
    # whose rounding moves max |C| (the deformation limit, not the governing
    # one here) by a few 1e-4
    _limits_close(gpu.time_step_limits(), lim_ref, rel=1e-3)
    out, exp = gpu.download(), ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=dx)
    if sort_interval == 8:
        assert gpu.stats()["sorts"] < done  # not every substep
    gpu.close()


def test_long_adaptive_run_replays_period_graphs(cuda_lib, oracle_mod):
    """Forty-odd adaptive substeps in the fused form: after the first batch
    the binning periods replay CUDA graphs (every step and redo flag lives on
    the device), and the run still matches the oracle substep for substep."""
    s = scenes.small_mixed()
    target, max_dt = 0.01, 2.5e-4
    gpu = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=4))
    status, done, t = gpu.step_adaptive(target, max_dt, s.gravity, time=0.0)
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=False)
    rc, n_ref, t_ref, lim_ref = ref.step_adaptive(0.0, target, max_dt, s.gravity)
    assert (status, rc) == (0, 0)
    assert done == n_ref and done >= 40
    assert abs(t - t_ref) <= 1e-5 * t_ref
    assert gpu.stats()["graph_replays"] > 0 and gpu.stats()["adaptive_split"] == 0
    # after forty substeps max |v| and max |C| carry the state's rounding
    # differences (velocities agree to the 1e-3 of TOL), so the velocity and
    # deformation limits are compared at that level
    _limits_close(gpu.time_step_limits(), lim_ref, rel=1e-3)
    out, exp = gpu.download(), ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=s.consts.grid_node_size)
    gpu.close()


def test_velocity_governed_run_falls_back_to_the_split_form(cuda_lib, oracle_mod):
    """Particles speeding up under strong gravity: the velocity limit shrinks
    every substep, so the fused form's speculative steps keep failing and
    the run moves to the split form after its first batch.  Both forms'
    substeps together match the oracle's."""
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.velocities[:] = np.array([20.0, 0.0, 0.0], np.float32)
    p.velocity_gradients[:] = 0
    g = (2000.0, 0.0, 0.0)
    target, max_dt = 0.02, 1e-2
    gpu = CudaState.from_io_state(IoState(0.0, p), s.consts)
    status, done, t = gpu.step_adaptive(target, max_dt, g, time=0.0)
    ref = oracle_mod.OracleState(p, s.consts, None, fp64=False)
    rc, n_ref, t_ref, lim_ref = ref.step_adaptive(0.0, target, max_dt, g)
    assert (status, rc) == (0, 0)
    assert done == n_ref and done > 16
    assert abs(t - t_ref) <= 1e-5 * t_ref
    lim = gpu.time_step_limits()
    assert lim["velocity"] < min(lim["sound"], lim["isolated"], lim["deformation"])
    # the governing velocity limit and the steps as tightly as everywhere;
    # max |C| of a body moving at 60 m/s is a small difference of large
    # terms, so the (non-governing) deformation limit only to 1e-2
    deformation = lim["deformation"]
    lim["deformation"] = float(lim_ref[4])
    _limits_close(lim, lim_ref)
    assert abs(deformation - lim_ref[4]) <= 1e-2 * lim_ref[4]
    st = gpu.stats()
    assert st["adaptive_misses"] > 0 and st["adaptive_split"] > 0
    out, exp = gpu.download(), ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=s.consts.grid_node_size)
    gpu.close()
