"""Batched scenes (an addition; the reference backend holds one scene):
several independent scenes in one handle must give each scene the result it
gets alone, culled against its own domain, through the C ABI."""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, InputConsts, IoState, scenes
from squishy_volumes_gb300.state import BatchedCudaState
from squishy_volumes_gb300._abi import SV_TOMBSTONED

pytestmark = pytest.mark.gpu


def _scenes():
    out = []
    for i, kind in enumerate(["neo_hookean", "sand", "snow", "fixed_corotated"]):
        s = scenes.small_mixed(n_per_material=64, seed=20 + i)
        # keep one material per scene, as the batched configuration does
        p = s.io_state.particles
        n = p.n // 6
        sub = p.subset(slice(i * n, (i + 1) * n))
        sub.velocities[:] = np.array([0.4 - 0.2 * i, 0.1 * i, -0.3], np.float32)
        lo = 0.1 * i
        consts = InputConsts(grid_node_size=s.consts.grid_node_size, domain_min=(lo, 0.0, 0.29 + 0.002 * i),
                             domain_max=(1.5, 1.5, 1.5))
        out.append((IoState(0.0, sub), consts))
    return out


def test_batched_scenes_match_single_runs(cuda_lib, oracle_mod):
    sc = _scenes()
    dt, g, n = 1e-4, (0.0, 0.0, -9.81), 8
    ext = Extras(position_form=1)
    b = BatchedCudaState.from_scenes([s for s, _ in sc], [c for _, c in sc], ext)
    assert b.scene_count() == len(sc)
    assert b.step(n, dt, g) == (0, n)
    for k, (io, consts) in enumerate(sc):
        got = b.download_scene(k)
        alone = CudaState.from_io_state(io, consts, ext)
        alone.step(n, dt, g)
        exp = alone.download()
        alone.close()
        np.testing.assert_array_equal(got.flags, exp.flags)
        for f, tol in [("positions", 1e-6), ("velocities", 1e-5), ("position_gradients", 1e-5)]:
            a, e = getattr(got, f).astype(np.float64), getattr(exp, f).astype(np.float64)
            assert np.linalg.norm(a - e) <= tol * np.linalg.norm(e) + 1e-9, (k, f)
        # and against the fp64 oracle of the scene alone (cull included)
        ref = oracle_mod.OracleState(io.particles, consts, None, fp64=True)
        ref.step(n, dt, g)
        o = ref.download()
        np.testing.assert_array_equal(got.flags, o.flags)
        live = (o.flags & SV_TOMBSTONED) == 0
        a, e = got.positions[live].astype(np.float64), o.positions[live].astype(np.float64)
        assert np.linalg.norm(a - e) <= 1e-6 * np.linalg.norm(e), k
    # the per-scene domains differ: scenes 1.. cull some particles at x > lo
    whole = b.download()
    assert whole.n == sum(io.particles.n for io, _ in sc)
    b.close()


def test_batched_64_configuration_builds_and_steps(cuda_lib):
    """The 64-scene configuration (~7.5M particles, lognormal sizes) runs a
    few substeps and conserves the particle count."""
    sc = scenes.batched_64()
    b = BatchedCudaState.from_scenes([s.io_state for s in sc], [s.consts for s in sc], sc[0].extras)
    assert b.step(4, sc[0].dt, sc[0].gravity) == (0, 4)
    st = b.stats()
    assert st["particles"] == sum(s.io_state.particles.n for s in sc)
    small = min(range(len(sc)), key=lambda i: sc[i].io_state.particles.n)
    out = b.download_scene(small)
    assert np.all(np.isfinite(out.positions))
    # a box landing on nothing in four substeps stays above its ground plane
    assert out.positions[:, 2].min() > sc[small].extras.ground_height
    b.close()
