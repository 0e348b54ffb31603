"""The reference's own literal test inputs through the GPU path.

tests/golden/reference_tables.npz holds, read from the reference's test
source by tests/golden/make_reference_tables.py:
  - the 512-point lattice of many_positions() (rust/crates/gpu/src/
    test_util.rs:112-631), which the reference's scatter, collect and step
    tests place at grid_node_size 0.5 (gpu/src/scatter/test.rs:93-140);
  - the 512 positions of specific_positions_and_collider_bits() (:678-2729)
    of its register_contributors, prepare_grid and step tests;
  - test_position_gradients_simple() (:633-676) and the parameter sets of
    test_lame_parameters / test_inviscid_parameters (util/src/elastic.rs:
    679-693), including the (E, nu) = (0, 0.4) solid with mu = 0.
The reference draws its velocities and random gradients from ChaCha8 (seed
42) through the rand crate; those draws are regenerated here with numpy's
seeded generator.  Each table goes through sv_p2g_only and one whole
substep, against the fp64 oracle: node sets exact, masses and velocities and
the particle state by norm (the reference's own check_iters_by_norm,
gpu/src/test_util.rs:2738-2764, uses 1e-6 + 1 % of the norm; ours are
tighter, stated per field).
"""

from pathlib import Path

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, InputConsts, IoState, Particles, scenes
from squishy_volumes_gb300._abi import SV_IS_FLUID, SV_IS_SOLID, SV_TOMBSTONED, SV_USE_SAND_ALPHA

pytestmark = pytest.mark.gpu

TABLES = np.load(Path(__file__).parent / "golden" / "reference_tables.npz")
DX = 0.5      # grid_node_size of the reference's scatter / collect tests
DT = 1e-3     # their time_step
RHO = 1000.0


def table_particles(positions: np.ndarray, seed: int, sand: bool = False) -> Particles:
    """Particles at the table's positions, cycling through the reference's
    Lame and inviscid parameter sets like its scatter test
    (parameters ... .cycle().take(n)), with seeded velocities, velocity
    gradients and deformation gradients (the simple table, then random
    near-identity ones)."""
    rng = np.random.default_rng(seed)
    n = len(positions)
    lame = TABLES["lame_parameters"]
    inv = TABLES["inviscid_parameters"]
    kinds = [("solid", e, nu) for e, nu in lame] + [("fluid", k, int(g)) for k, g in inv]
    flags = np.zeros(n, np.uint32)
    mu = np.zeros(n, np.float32)
    lam = np.zeros(n, np.float32)
    bulk = np.zeros(n, np.float32)
    expo = np.zeros(n, np.int32)
    alpha = np.zeros(n, np.float32)
    for i in range(n):
        kind, a, b = kinds[i % len(kinds)]
        if kind == "solid":
            flags[i] = SV_IS_SOLID
            mu[i], lam[i] = scenes.lame(a, b)
            if sand:
                flags[i] |= SV_USE_SAND_ALPHA
                alpha[i] = scenes.friction_angle_to_alpha(np.deg2rad(30.0))
        else:
            flags[i] = SV_IS_FLUID
            bulk[i], expo[i] = a, b
    simple = TABLES["simple_gradients"]
    F = np.empty((n, 9), np.float32)
    for i in range(n):
        if i < len(simple) * 8:
            F[i] = simple[i % len(simple)]
        else:
            F[i] = (np.eye(3) + rng.uniform(-0.05, 0.05, (3, 3))).T.reshape(9)
    vol = np.full(n, (DX / 2) ** 3, np.float32)
    return Particles(
        flags=flags,
        positions=positions.astype(np.float32),
        position_gradients=F,
        velocities=rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32),
        velocity_gradients=rng.uniform(-1.0, 1.0, (n, 9)).astype(np.float32),
        mass=(vol * RHO).astype(np.float32),
        initial_volume=vol,
        mu=mu,
        lambda_=lam,
        sand_alpha=alpha if sand else None,
        exponent=expo,
        bulk_modulus=bulk,
    )


def table_consts(positions: np.ndarray) -> InputConsts:
    lo = positions.min(0) - 4 * DX
    hi = positions.max(0) + 4 * DX
    return InputConsts(grid_node_size=DX, domain_min=tuple(float(x) for x in lo), domain_max=tuple(float(x) for x in hi))


@pytest.mark.parametrize("table", ["many_positions", "specific_positions"])
def test_reference_table_p2g_matches_oracle(cuda_lib, oracle_mod, table):
    pos = TABLES[table]
    p = table_particles(pos, seed=42)
    consts = table_consts(pos)
    gravity = (0.0, 0.0, -9.81)
    gpu = CudaState.from_io_state(IoState(0.0, p), consts)
    g = gpu.p2g_only(DT, gravity)
    st = gpu.stats()
    gpu.close()
    ref = oracle_mod.OracleState(p, consts, None, fp64=True)
    ref.p2g_only(DT, gravity)
    ids, m, v = ref.grid()
    ref.close()
    np.testing.assert_array_equal(g.node_ids, ids)
    np.testing.assert_allclose(g.masses, m, rtol=4e-6, atol=1e-6 * float(p.mass.max()))
    err = np.linalg.norm(g.velocities.astype(np.float64) - v) / np.linalg.norm(v)
    assert err <= 1e-5, err
    # the device's fp64 conservation sums of the same grid
    np.testing.assert_allclose(st["grid_mass"], p.mass.sum(dtype=np.float64), rtol=1e-6)


@pytest.mark.parametrize("table", ["many_positions", "specific_positions"])
@pytest.mark.parametrize("sand", [False, True])
def test_reference_table_substep_matches_oracle(cuda_lib, oracle_mod, table, sand):
    """One whole substep; with `sand` every solid takes the Drucker-Prager
    return map, the (E, nu) = (0, 0.4) ones with mu = 0 included: the
    table's gradients are rotations and stretches (expansion, e_tr >= 0), the
    branch where the reference projects F to U V^T whatever mu is."""
    pos = TABLES[table]
    p = table_particles(pos, seed=7, sand=sand)
    if sand:
        # expansions only (the simple table's rotations and stretches, scaled
        # by 1.03: det F >= 1.09, which one substep's F += dt C F cannot bring
        # below 1); the compressive branch with mu = 0 is the reference's
        # assert, tested on its own in test_gpu_parity.py
        simple = TABLES["simple_gradients"]
        p.position_gradients[:] = 1.03 * simple[np.arange(p.n) % len(simple)]
    consts = table_consts(pos)
    gravity = (0.0, 0.0, -9.81)
    gpu = CudaState.from_io_state(IoState(0.0, p), consts)
    assert gpu.step(1, DT, gravity) == (0, 1)
    out = gpu.download()
    gpu.close()
    ref = oracle_mod.OracleState(p, consts, None, fp64=True)
    assert ref.step(1, DT, gravity) == 0
    exp = ref.download()
    ref.close()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    for name, rel in (("positions", 1e-6), ("velocities", 1e-4), ("position_gradients", 2e-5),
                      ("velocity_gradients", 1e-3)):
        a = getattr(out, name)[live].astype(np.float64)
        b = getattr(exp, name)[live].astype(np.float64)
        err = np.linalg.norm(a - b)
        assert err <= 1e-6 + rel * np.linalg.norm(b), (name, err / np.linalg.norm(b))
