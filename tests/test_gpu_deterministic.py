"""The deterministic P2G mode (sv_consts.deterministic_p2g = 1).

Grid mass must match exactly the fp32 rounding of a deterministic
segmented sum.  The reference sums each node's
contributions in whatever order its contributor lists were filled under a
mutex (rust/crates/cpu/src/phase/update_grid_nodes.rs:101-122), so its
result is not reproducible; the oracle's svo_deterministic_grid_mass fixes
one order -- the 27 base cells around the node in lexicographic order, each
cell's particles in ascending original index -- and sums the reference's
per-pair mass (scatter_momentum.rs:22-93, kernels.rs:17-26) left to right in
fp32.  In this mode the GPU must produce those node masses bit for bit, and
two runs of the same input must give the same bits everywhere.
"""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, IoState, scenes
from squishy_volumes_gb300._abi import SV_TOMBSTONED, SvError
from test_gpu_parity import compare_states

pytestmark = pytest.mark.gpu


def det(extras):
    """The scene's options with the deterministic P2G (fp32 positions)."""
    d = dict(extras.__dict__) if extras is not None else {}
    d.update(deterministic_p2g=1, position_form=0)
    return Extras(**d)


def _grid_vs_oracle(oracle_mod, io_state, consts, extras, dt, gravity):
    gpu = CudaState.from_io_state(io_state, consts, det(extras))
    g = gpu.p2g_only(dt, gravity)
    gpu.close()
    p = io_state.particles
    ids, m = oracle_mod.deterministic_grid_mass(p.positions, p.mass, p.flags, consts.grid_node_size)
    np.testing.assert_array_equal(g.node_ids, ids)
    # bit for bit
    np.testing.assert_array_equal(g.masses.view(np.uint32), m.view(np.uint32))


@pytest.mark.parametrize("scene", ["small_mixed", "cube_64k", "three_boxes_1m"])
def test_deterministic_grid_mass_is_bit_exact(cuda_lib, oracle_mod, scene):
    s = scenes.SCENES[scene]()
    _grid_vs_oracle(oracle_mod, s.io_state, s.consts, s.extras, s.dt, s.gravity)


def test_deterministic_grid_mass_after_dynamics(cuda_lib, oracle_mod):
    """The same after 15 substeps of the mode (particles moved, deformed,
    jittered out of their initial lattice)."""
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, det(s.extras))
    assert gpu.step(15, s.dt, s.gravity) == (0, 15)
    state = gpu.download()
    gpu.close()
    _grid_vs_oracle(oracle_mod, IoState(0.0, state), s.consts, s.extras, s.dt, s.gravity)


def test_deterministic_runs_are_bitwise_reproducible(cuda_lib, oracle_mod):
    s = scenes.cube_64k()
    outs = []
    for _ in range(2):
        gpu = CudaState.from_io_state(s.io_state, s.consts, det(s.extras))
        assert gpu.step(12, s.dt, s.gravity) == (0, 12)
        outs.append(gpu.download())
        gpu.close()
    a, b = outs
    for k in ("flags", "positions", "velocities", "velocity_gradients", "position_gradients", "elastic_energies"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    # and it is the same physics: the fp64 oracle within the usual tolerances
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, s.extras, fp64=True)
    assert ref.step(12, s.dt, s.gravity) == 0
    exp = ref.download()
    ref.close()
    np.testing.assert_array_equal(a.flags, exp.flags)
    compare_states(a, exp, (exp.flags & SV_TOMBSTONED) == 0, dx=s.consts.grid_node_size)


def test_deterministic_mode_needs_fp32_positions(cuda_lib):
    s = scenes.small_mixed()
    with pytest.raises(SvError, match="deterministic_p2g"):
        CudaState.from_io_state(s.io_state, s.consts, Extras(deterministic_p2g=1, position_form=1))
