"""CUDA-graph replay of binning periods and the launch autotuner.

A binning period (the binning substep and the substeps up to the next
binning) is captured once per launch configuration and replayed; the replay
must give what launching the same kernels one by one gives, and both must
match the oracle.  The autotuner times candidate configurations on a
snapshot of the state and must hand the state back unchanged.
"""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, scenes
from squishy_volumes_gb300._abi import SV_TOMBSTONED

from test_gpu_parity import compare_states

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", [0, 1])
def test_graph_replay_matches_direct_launches(cuda_lib, oracle_mod, form):
    s = scenes.small_mixed()
    n = 40
    graphs = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=4, position_form=form))
    direct = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=4, position_form=form))
    direct.set_graphs(False)
    assert graphs.step(n, s.dt, s.gravity) == (0, n)
    assert direct.step(n, s.dt, s.gravity) == (0, n)
    sg, sd = graphs.stats(), direct.stats()
    assert sg["graph_replays"] > 0
    assert sd["graph_replays"] == 0
    assert sg["sorts"] == sd["sorts"]
    assert sg["kernel_launches"] == sd["kernel_launches"]
    a, b = graphs.download(), direct.download()
    np.testing.assert_array_equal(a.flags, b.flags)
    live = (b.flags & SV_TOMBSTONED) == 0
    # same kernels in the same order: only float-atomic summation order differs
    tight = {"positions": 1e-6, "velocities": 1e-5, "position_gradients": 1e-6}
    compare_states(a, b, live, tol=tight)
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=True)
    assert ref.step(n, s.dt, s.gravity) == 0
    exp = ref.download()
    np.testing.assert_array_equal(a.flags, exp.flags)
    compare_states(a, exp, live, tol={"positions": 1e-5, "velocities": 1e-3, "position_gradients": 1e-4},
                   dx=s.consts.grid_node_size)
    graphs.close(), direct.close()


@pytest.mark.parametrize("form", [0, 1])
def test_partial_periods_replay_like_direct_launches(cuda_lib, form):
    """Calls of 3 substeps with binning every 4 cut every binning period:
    each call replays the rest of one period and the start of the next as
    graphs keyed by where the period stands (captured when a part recurs).
    The result must be what launching the same kernels one by one gives."""
    s = scenes.small_mixed()
    calls, k = 20, 3
    graphs = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=4, position_form=form))
    direct = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=4, position_form=form))
    direct.set_graphs(False)
    for _ in range(calls):
        assert graphs.step(k, s.dt, s.gravity) == (0, k)
        assert direct.step(k, s.dt, s.gravity) == (0, k)
    sg, sd = graphs.stats(), direct.stats()
    assert sg["substeps"] == sd["substeps"] == calls * k
    # no call holds a whole period, so every replay is of a part of one;
    # the host state repeats every 8 calls, so parts recur within 20
    assert sg["graph_replays"] > 0
    assert sg["sorts"] == sd["sorts"]
    assert sg["kernel_launches"] == sd["kernel_launches"]
    a, b = graphs.download(), direct.download()
    np.testing.assert_array_equal(a.flags, b.flags)
    live = (b.flags & SV_TOMBSTONED) == 0
    compare_states(a, b, live, tol={"positions": 1e-6, "velocities": 1e-5, "position_gradients": 1e-6})
    graphs.close(), direct.close()


def test_graphs_follow_changing_inputs(cuda_lib):
    """A new dt or gravity is a new graph: the result still follows the
    inputs of each call."""
    s = scenes.small_mixed()
    a = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=2))
    b = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=2))
    b.set_graphs(False)
    for g in (s.gravity, (0.0, 0.0, 0.0), s.gravity):
        for st in (a, b):
            assert st.step(8, s.dt, g) == (0, 8)
        for st in (a, b):
            assert st.step(8, s.dt * 0.5, g) == (0, 8)
    ra, rb = a.download(), b.download()
    live = (rb.flags & SV_TOMBSTONED) == 0
    compare_states(ra, rb, live, tol={"positions": 1e-6, "velocities": 1e-5})
    assert a.stats()["graph_replays"] > 0
    a.close(), b.close()


def test_autotune_restores_state_and_keeps_parity(cuda_lib, oracle_mod):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts)
    before = gpu.download()
    choice = gpu.autotune(s.dt, s.gravity, 8)
    assert choice["sort_interval"] in (1, 2, 4, 6, 8, 12, 16)
    assert choice["cta_per_sm"] in (8, 16, 32, 64, 128)
    st = gpu.stats()
    assert st["sort_interval"] == choice["sort_interval"]
    assert st["cta_per_sm"] == choice["cta_per_sm"]
    assert st["substeps"] == 0
    after = gpu.download()
    for name in ("flags", "positions", "velocities", "velocity_gradients", "position_gradients"):
        np.testing.assert_array_equal(getattr(after, name), getattr(before, name), err_msg=name)
    assert gpu.step(s.substeps, s.dt, s.gravity) == (0, s.substeps)
    out = gpu.download()
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=True)
    assert ref.step(s.substeps, s.dt, s.gravity) == 0
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, dx=s.consts.grid_node_size)
    gpu.close()
