"""The frame cache storing a handle's state (sv_cache_store): the queued
copy must capture the state at the store even though the handle keeps
stepping, and the written frame must equal what sv_download /
sv_download_grid give at that point (to_io_state), with the parameters and
initial positions from the statics.  With colliders the grid entries carry
their collider bits (the reference's GridKey variants)."""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, IoState, scenes
from squishy_volumes_gb300.frames import FrameCache, read_frame

pytestmark = pytest.mark.gpu

STATIC = ["mass", "initial_volume", "exponent", "bulk_modulus"]
DYNAMIC = ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "elastic_energies",
           "collider_bits"]


def check_frame(frame: IoState, expected: IoState, statics, grid_expected=None):
    assert frame.time == expected.time
    for k in DYNAMIC:
        np.testing.assert_array_equal(getattr(frame.particles, k), getattr(expected.particles, k), err_msg=k)
    for k in STATIC:
        np.testing.assert_array_equal(getattr(frame.particles, k), getattr(statics, k), err_msg=k)
    x0 = statics.initial_positions if statics.initial_positions is not None else statics.positions
    np.testing.assert_array_equal(frame.particles.initial_positions, x0)
    if grid_expected is not None:
        g = frame.grid_nodes
        plain = g.collider_bits == 0
        np.testing.assert_array_equal(g.node_ids[plain], grid_expected.node_ids)
        np.testing.assert_array_equal(g.masses[plain], grid_expected.masses)
        np.testing.assert_array_equal(g.velocities[plain], grid_expected.velocities)
        # sorted by node id, then collider bits
        keys = [tuple(i) + (int(b),) for i, b in zip(g.node_ids, g.collider_bits)]
        assert keys == sorted(keys)


@pytest.mark.parametrize("form,depth", [(0, 2), (1, 1)])
def test_store_while_stepping(cuda_lib, tmp_path, form, depth):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, Extras(position_form=form))
    expected = []
    with FrameCache(tmp_path, s.io_state.particles, depth=depth) as cache:
        for k in range(4):
            assert gpu.step(15, s.dt, s.gravity)[0] == 0
            gpu_grid = gpu.grid()
            expected.append((gpu.to_io_state(store_grid=False), gpu_grid))
            cache.store(gpu, store_grid=k % 2 == 0)
        # the handle keeps stepping while the writer works
        assert gpu.step(15, s.dt, s.gravity)[0] == 0
        cache.flush()
        assert cache.info()[0] == 4
    for k, (io, grid) in enumerate(expected):
        frame = read_frame(tmp_path / f"frame_{k:05d}.bin")
        assert (frame.grid_nodes is not None) == (k % 2 == 0)
        check_frame(frame, io, s.io_state.particles, grid if k % 2 == 0 else None)
    gpu.close()


def test_store_with_collider_variants(cuda_lib, oracle_mod, tmp_path):
    from test_gpu_colliders import _consts, _falling_box, _frame, _quad

    p = _falling_box()
    consts = _consts()
    V, T, col = _quad(0.45)
    gpu = CudaState.from_io_state(IoState(0.0, p), consts, Extras())
    gpu.set_frame_input(_frame(V=V, T=T, col=col))
    with FrameCache(tmp_path, p) as cache:
        assert gpu.step(300, 1e-4, (0, 0, 0)) == (0, 300)
        expected, grid = gpu.to_io_state(store_grid=False), gpu.grid()
        cache.store(gpu, store_grid=True)
        cache.flush()
    frame = read_frame(tmp_path / "frame_00000.bin")
    check_frame(frame, expected, p, grid)
    assert (frame.particles.collider_bits != 0).any()
    assert (frame.grid_nodes.collider_bits != 0).any()  # the near-collider variants
    gpu.close()
