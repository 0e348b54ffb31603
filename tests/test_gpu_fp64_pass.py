"""The fused pass's fp64 pass, against the fp64 oracle.

The plain fused particle pass carries no fp64 SVD code.  A particle whose
fp32 SVD is degenerate, or that the fp64 policy flags (policy 1: det F <
0.05; policy 2 also: two singular values closer than 1e-4), is left out of
the fused pass and listed; a second pass then runs that particle's whole
substep again from the same input state and grid with the fp64 SVD, its
gather and scatter through global memory.  The listed particles must end up
like every other particle: within the parity tolerances of the fp64 oracle,
and counted as fp64 SVDs.
"""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, IoState, scenes
from squishy_volumes_gb300._abi import SV_IS_FLUID, SV_TOMBSTONED

from test_gpu_parity import compare_states

pytestmark = pytest.mark.gpu


def _rotations(rng, k):
    q = rng.normal(size=(k, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def _run(particles, scene, policy, substeps):
    gpu = CudaState.from_io_state(IoState(0.0, particles), scene.consts, Extras(svd_fp64_policy=policy))
    assert gpu.step(substeps, scene.dt, scene.gravity) == (0, substeps)
    out, fp64 = gpu.download(), gpu.stats()["fp64_svd"]
    gpu.close()
    return out, fp64


def _compressed(n_per_material, fraction, seed=7):
    """small_mixed with a share of its solid particles compressed to
    det F = 0.042: a rotated diag(0.3, 0.35, 0.4)."""
    s = scenes.small_mixed(n_per_material=n_per_material)
    p = s.io_state.particles.copy()
    rng = np.random.default_rng(seed)
    solids = np.flatnonzero((p.flags & SV_IS_FLUID) == 0)
    pick = rng.choice(solids, max(1, int(solids.size * fraction)), replace=False)
    F = _rotations(rng, pick.size) @ np.diag([0.3, 0.35, 0.4])[None]
    p.position_gradients[pick] = F.transpose(0, 2, 1).reshape(-1, 9).astype(np.float32)  # column-major
    return s, p, pick


@pytest.mark.parametrize("policy", [0, 1])
def test_compressed_solids_take_the_fp64_pass(cuda_lib, oracle_mod, policy):
    """A tenth of the solid particles start compressed below det F = 0.05:
    policy 1 sends them through the fp64 pass every substep they stay there,
    policy 0 keeps them in the fp32 fused pass.  Both must match the fp64
    oracle; only policy 1 counts fp64 SVDs."""
    s, p, pick = _compressed(1000, 0.1)
    substeps = 3
    out, fp64 = _run(p, s, policy, substeps)
    ref = oracle_mod.OracleState(p, s.consts, s.extras, fp64=True)
    assert ref.step(substeps, s.dt, s.gravity) == 0
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, dx=s.consts.grid_node_size)
    if policy == 0:
        assert fp64 == 0
    else:
        assert fp64 >= pick.size, (fp64, pick.size)


def test_many_listed_particles_spread_over_the_fp64_pass(cuda_lib, oracle_mod):
    """Every solid particle compressed (about 20k of 29k stay below det F =
    0.05 for the whole run): more listed particles per substep than the fp64
    pass has threads, so its CTAs take several chunks each."""
    s, p, pick = _compressed(5000, 1.0)
    assert pick.size > 20_000
    substeps = 4
    out, fp64 = _run(p, s, 1, substeps)
    ref = oracle_mod.OracleState(p, s.consts, s.extras, fp64=True)
    assert ref.step(substeps, s.dt, s.gravity) == 0
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, dx=s.consts.grid_node_size)
    assert fp64 >= 2 * pick.size, (fp64, pick.size)


def test_listed_particles_in_graph_replays(cuda_lib, oracle_mod):
    """With a tenth of the solids compressed (listed for the fp64 pass every
    substep under policy 1) and whole binning periods replayed as CUDA
    graphs, the run must match the fp64 oracle like the same kernels
    launched one by one, with the same fp64 count.  (Graph and direct runs
    differ from each other by float-atomic order in the scatter only: 3e-5
    in the velocities of these stiff particles.)"""
    s, p, _ = _compressed(1000, 0.1)
    ex = Extras(svd_fp64_policy=1, sort_interval=4)
    calls, k = 3, 4
    graphs = CudaState.from_io_state(IoState(0.0, p), s.consts, ex)
    direct = CudaState.from_io_state(IoState(0.0, p), s.consts, ex)
    direct.set_graphs(False)
    for _ in range(calls):
        assert graphs.step(k, s.dt, s.gravity) == (0, k)
        assert direct.step(k, s.dt, s.gravity) == (0, k)
    sg, sd = graphs.stats(), direct.stats()
    assert sg["graph_replays"] > 0 and sd["graph_replays"] == 0
    assert sg["substeps"] == sd["substeps"] == calls * k
    assert sg["fp64_svd"] == sd["fp64_svd"] > 0
    ref = oracle_mod.OracleState(p, s.consts, ex, fp64=True)
    assert ref.step(calls * k, s.dt, s.gravity) == 0
    exp = ref.download()
    live = (exp.flags & SV_TOMBSTONED) == 0
    for st in (graphs, direct):
        out = st.download()
        np.testing.assert_array_equal(out.flags, exp.flags)
        compare_states(out, exp, live, dx=s.consts.grid_node_size)
    graphs.close(), direct.close()
