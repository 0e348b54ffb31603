"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances: integer and index work (binning keys, sort permutation, node
sets, flags) must match bit for bit.  Floating-point results are compared by
norm like the reference's check_iters_by_norm (rust/crates/gpu/src/
test_util.rs:2738-2764: error <= 1e-6 + rel * |b|), with rel stated per field
below; summation order differs between the two (float atomics on the GPU,
node-ordered gathers on the CPU), so bit equality is not expected.
"""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, InputConsts, IoState, scenes, sort_pairs
from squishy_volumes_gb300._abi import SV_FAILED, SV_IS_SOLID, SV_STATUS_PARTICLE_INVERTED, SV_TOMBSTONED, SvError

pytestmark = pytest.mark.gpu

# Relative tolerances (by norm) per field after a few substeps.
TOL = {
    "positions": 1e-6,
    "velocities": 1e-4,
    "velocity_gradients": 1e-3,
    "position_gradients": 1e-5,
    "elastic_energies": 1e-3,
}


def by_norm(a, b, rel, eps=1e-6):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    err = np.linalg.norm(a - b)
    scale = max(np.linalg.norm(a), np.linalg.norm(b))
    return err <= eps + rel * scale, err / max(scale, 1e-30)


def compare_states(gpu, ref, live, tol=TOL, dx=None):
    for name, rel in tol.items():
        a = getattr(gpu, name)[live]
        b = getattr(ref, name)[live]
        if name == "velocity_gradients" and dx is not None:
            # C ~ |v| / dx is its natural scale: in a rigid motion C vanishes
            # analytically and both sides hold only rounding noise.
            a64, b64 = a.astype(np.float64), b.astype(np.float64)
            scale = max(np.linalg.norm(b64), np.linalg.norm(ref.velocities[live].astype(np.float64)) / dx)
            r = np.linalg.norm(a64 - b64) / max(scale, 1e-30)
            assert r <= rel, f"{name}: error {r:.3e} of max(|C|, |v|/dx) > {rel}"
            continue
        if name == "elastic_energies":
            # Near rest the energy is second order in fp32 noise of F
            # (psi ~ modulus * eps^2): floor the scale at modulus * 1e-10 per particle.
            a64, b64 = a.astype(np.float64), b.astype(np.float64)
            modulus = max(float(np.max(np.abs(ref.mu[live]))) if ref.mu is not None else 0.0,
                          float(np.max(np.abs(ref.lambda_[live]))) if ref.lambda_ is not None else 0.0,
                          float(np.max(np.abs(ref.bulk_modulus[live]))) if ref.bulk_modulus is not None else 0.0)
            scale = max(np.linalg.norm(b64), modulus * 1e-10 * np.sqrt(max(len(b64), 1)))
            r = np.linalg.norm(a64 - b64) / max(scale, 1e-30)
            assert r <= rel, f"{name}: error {r:.3e} of max(|E|, modulus 1e-10 sqrt(n)) > {rel}"
            continue
        ok, r = by_norm(a, b, rel)
        assert ok, f"{name}: relative error {r:.3e} > {rel}"


# ---------------------------------------------------------------- sort
@pytest.mark.parametrize("n", [0, 1, 2, 1000, 4097, 100_000])
def test_sort_pairs_is_stable_sort(cuda_lib, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 50, n).astype(np.uint32)  # many duplicates
    perm = sort_pairs(keys)
    np.testing.assert_array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))


@pytest.mark.parametrize("key_bits", [1, 9, 10, 17, 20, 25, 28, 30])
def test_sort_pairs_digit_widths(cuda_lib, key_bits):
    # the passes split the significant bits evenly into digits of at most
    # 10 bits: 25 bits sort as 9 + 8 + 8, 28 as 10 + 9 + 9, 17 as 9 + 8
    rng = np.random.default_rng(key_bits)
    keys = rng.integers(0, 2**key_bits, 150_000, dtype=np.uint64).astype(np.uint32)
    keys[::5] = keys[::5] >> (key_bits // 2)  # duplicates and short keys
    keys[3] = 2**key_bits - 1
    perm = sort_pairs(keys)
    np.testing.assert_array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))


def test_sort_pairs_all_zero_keys(cuda_lib):
    perm = sort_pairs(np.zeros(5000, np.uint32))
    np.testing.assert_array_equal(perm, np.arange(5000, dtype=np.uint32))


def test_sort_pairs_full_32_bit_keys(cuda_lib):
    rng = np.random.default_rng(42)
    keys = rng.integers(0, 2**32, 300_000, dtype=np.uint64).astype(np.uint32)
    keys[::7] = 0xFFFFFFFF
    perm = sort_pairs(keys)
    np.testing.assert_array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))


# ---------------------------------------------------------------- binning
def test_binning_keys_and_permutation_match_cpu(cuda_lib, oracle_mod):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    origin, nb = gpu.grid_layout()
    keys, perm, orig = gpu.binning()
    p = s.io_state.particles
    exp = oracle_mod.binning_keys(p.positions[orig], p.flags[orig], s.consts.grid_node_size, origin, nb)
    np.testing.assert_array_equal(keys, exp)
    np.testing.assert_array_equal(perm, oracle_mod.stable_sort_perm(exp))
    # after substeps the keys come from the G2P epilogue of the last substep
    gpu.step(3, s.dt, s.gravity)
    keys, perm, orig = gpu.binning()
    cur = gpu.download()
    exp = oracle_mod.binning_keys(cur.positions[orig], cur.flags[orig], s.consts.grid_node_size, origin, nb)
    np.testing.assert_array_equal(keys, exp)
    np.testing.assert_array_equal(perm, oracle_mod.stable_sort_perm(exp))
    # keys are the reference's lexicographic cell order refined to 4^3 blocks:
    # after a substep the device order is sorted by the previous keys
    assert np.all(np.diff(keys[perm].astype(np.int64)) >= 0)
    gpu.close()


# ---------------------------------------------------------------- P2G / grid
@pytest.mark.parametrize("fp64", [False, True])
def test_p2g_grid_matches_oracle(cuda_lib, oracle_mod, fp64):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    g = gpu.p2g_only(s.dt, s.gravity)
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, s.extras, fp64=fp64)
    ref.p2g_only(s.dt, s.gravity)
    ids, m, v = ref.grid()
    np.testing.assert_array_equal(g.node_ids, ids)
    # grid mass: fp32 sums of <= 216 positive terms in another order; nodes at
    # the stencil rim hold tiny weights whose own rounding dominates, hence the
    # absolute floor of 1e-6 of a particle mass
    m_p = float(s.io_state.particles.mass.max())
    np.testing.assert_allclose(g.masses, m, rtol=4e-6, atol=1e-6 * m_p)
    ok, r = by_norm(g.velocities, v, 1e-5)
    assert ok, r
    gpu.close()


def test_p2g_conserves_momentum(cuda_lib):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, Extras())
    g = gpu.p2g_only(s.dt, s.gravity)
    p = s.io_state.particles
    grid_mom = (g.masses[:, None].astype(np.float64) * g.velocities).sum(0)
    part_mom = (p.mass[:, None].astype(np.float64) * (p.velocities + s.dt * np.asarray(s.gravity, np.float32))).sum(0)
    scale = (p.mass.astype(np.float64)[:, None] * np.abs(p.velocities)).sum()
    assert np.all(np.abs(grid_mom - part_mom) <= 1e-6 * scale), (grid_mom, part_mom)
    np.testing.assert_allclose(g.masses.sum(dtype=np.float64), p.mass.sum(dtype=np.float64), rtol=1e-6)
    gpu.close()


# ---------------------------------------------------------------- whole substeps
def test_matches_committed_golden_vectors(cuda_lib):
    """The CUDA path against tests/golden/oracle_small_mixed.npz (fp64 oracle
    output committed with its generator, tests/golden/make_golden.py)."""
    from pathlib import Path

    from squishy_volumes_gb300 import Particles

    g = np.load(Path(__file__).parent / "golden" / "oracle_small_mixed.npz")
    names = ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "mass",
             "initial_volume", "mu", "lambda_", "sand_alpha", "exponent", "bulk_modulus", "viscosity_dynamic",
             "viscosity_bulk", "model", "hardening", "crit_compression", "crit_stretch", "plastic_j"]
    p = Particles(**{k: g[f"in_{k}"] for k in names})
    consts = InputConsts(grid_node_size=float(g["grid_node_size"]), domain_min=tuple(g["domain_min"]),
                         domain_max=tuple(g["domain_max"]))
    gpu = CudaState.from_io_state(IoState(0.0, p), consts)
    assert gpu.step(int(g["substeps"]), float(g["dt"]), g["gravity"]) == (0, int(g["substeps"]))
    out = gpu.download()

    class Ref:
        pass

    ref = Ref()
    for k in ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "elastic_energies",
              "plastic_j"]:
        setattr(ref, k, g[f"out_{k}"])
    ref.mu, ref.lambda_, ref.bulk_modulus = p.mu, p.lambda_, p.bulk_modulus
    np.testing.assert_array_equal(out.flags, ref.flags)
    live = (ref.flags & SV_TOMBSTONED) == 0
    compare_states(out, ref, live, dx=consts.grid_node_size)
    gpu.close()



@pytest.mark.parametrize("fp64,sort_interval", [(False, 0), (True, 0), (True, 1), (True, 3)])
def test_substeps_match_oracle(cuda_lib, oracle_mod, fp64, sort_interval):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, Extras(sort_interval=sort_interval))
    status, done = gpu.step(s.substeps, s.dt, s.gravity)
    assert (status, done) == (0, s.substeps)
    out = gpu.download()
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, s.extras, fp64=fp64)
    assert ref.step(s.substeps, s.dt, s.gravity) == 0
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, dx=s.consts.grid_node_size)
    # Snow's plastic J multiplies each substep's volume change, and its
    # hardening exp(10 (1 - J_p)) feeds back into the stress, so the float
    # atomics' summation order (which differs from run to run) moves single
    # particles by up to about 1e-5 against the fp32 oracle after these 10
    # substeps (1.04e-5 seen once in about 25 runs).
    np.testing.assert_allclose(out.plastic_j, exp.plastic_j, rtol=3e-5 if not fp64 else 1e-5)
    gpu.close()


def test_cube_64k_matches_fp64_oracle(cuda_lib, oracle_mod):
    s = scenes.cube_64k()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    n = 20
    assert gpu.step(n, s.dt, s.gravity) == (0, n)
    out = gpu.download()
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, s.extras, fp64=True)
    assert ref.step(n, s.dt, s.gravity) == 0
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    compare_states(out, exp, np.ones(out.n, bool), dx=s.consts.grid_node_size)
    gpu.close()


def test_cell_offset_positions_match_fp32_positions(cuda_lib, oracle_mod):
    s = scenes.small_mixed()
    a = CudaState.from_io_state(s.io_state, s.consts, Extras(position_form=0))
    b = CudaState.from_io_state(s.io_state, s.consts, Extras(position_form=1))
    a.step(s.substeps, s.dt, s.gravity)
    b.step(s.substeps, s.dt, s.gravity)
    ra, rb = a.download(), b.download()
    ref = oracle_mod.OracleState(s.io_state.particles, s.consts, None, fp64=True)
    ref.step(s.substeps, s.dt, s.gravity)
    exp = ref.download()
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(rb, exp, live, dx=s.consts.grid_node_size)
    # the cell form is at least as close to the fp64 oracle in position
    ea = np.linalg.norm(ra.positions[live].astype(np.float64) - exp.positions[live])
    eb = np.linalg.norm(rb.positions[live].astype(np.float64) - exp.positions[live])
    assert eb <= ea * 1.5 + 1e-12
    a.close(), b.close()


def test_split_calls_match_one_call(cuda_lib):
    """The scatter left pending at the end of a call is reused by the next
    call with the same dt and gravity, and redone when they differ."""
    s = scenes.small_mixed()
    one = CudaState.from_io_state(s.io_state, s.consts)
    two = CudaState.from_io_state(s.io_state, s.consts)
    three = CudaState.from_io_state(s.io_state, s.consts)
    one.step(10, s.dt, s.gravity)
    two.step(4, s.dt, s.gravity)
    two.step(6, s.dt, s.gravity)
    three.step(4, s.dt, (0.0, 0.0, 0.0))
    three.step(6, s.dt, s.gravity)
    a, b, c = one.download(), two.download(), three.download()
    compare_states(b, a, np.ones(a.n, bool), dx=s.consts.grid_node_size)
    # gravity differed for four substeps: velocities must differ
    assert not np.allclose(c.velocities, a.velocities)
    one.close(), two.close(), three.close()


def test_fast_particles_rebin(cuda_lib, oracle_mod):
    """Particles crossing several cells per substep leave their binning
    tiles and blocks; the result must still match the oracle."""
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    dx = s.consts.grid_node_size
    p.velocities[:] = np.array([1.5, -1.0, 0.7], np.float32) * (dx / s.dt)  # 1.5 cells per substep
    p.velocity_gradients[:] = 0
    io = IoState(0.0, p)
    gpu = CudaState.from_io_state(io, s.consts, Extras(sort_interval=8))
    assert gpu.step(6, s.dt, (0, 0, 0)) == (0, 6)
    out = gpu.download()
    ref = oracle_mod.OracleState(p, s.consts, None, fp64=True)
    ref.step(6, s.dt, (0, 0, 0))
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, dx=dx)
    gpu.close()


@pytest.mark.parametrize("form", [0, 1])
def test_free_fall_leaves_fluid_and_sand_unstrained(cuda_lib, oracle_mod, form):
    """Bodies at rest in free fall: the grid velocity is uniform, so C is
    rounding noise and F must stay the identity to that noise.  The fluid
    and sand returns rebuild F from U V^T every substep; an SVD that rotated
    columns already orthogonal to fp32 epsilon (F = I + 1e-13) put 1e-8
    noise into F there, which the stiff fluid turned into pressure."""
    from squishy_volumes_gb300.scenes import Material, build_particles, jittered_box
    from squishy_volumes_gb300 import IoState

    rng = np.random.default_rng(11)
    dx = 1.0 / 256
    blocks = [(jittered_box(rng, (0.3, 0.3, 0.3), (24, 24, 16), dx / 2), Material("fluid", bulk_modulus=1e5), (0, 0, 0),
               dx / 2),
              (jittered_box(rng, (0.5, 0.3, 0.3), (16, 16, 16), dx / 2), Material("sand", youngs_modulus=1e5), (0, 0, 0),
               dx / 2)]
    p = build_particles(blocks)
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
    n, dt, g = 10, 2e-5, (0.0, 0.0, -9.81)
    gpu = CudaState.from_io_state(IoState(0.0, p), consts, Extras(position_form=form))
    assert gpu.step(n, dt, g) == (0, n)
    out = gpu.download()
    gpu.close()
    eye = np.eye(3, dtype=np.float32).reshape(9)
    assert np.abs(out.position_gradients - eye).max() <= 1e-9
    np.testing.assert_allclose(out.velocities[:, 2], -9.81 * n * dt, rtol=1e-5)
    assert np.abs(out.velocities[:, :2]).max() <= 1e-9
    ref = oracle_mod.OracleState(p, consts, None, fp64=True)
    assert ref.step(n, dt, g) == 0
    exp = ref.download()
    ok, r = by_norm(out.velocities, exp.velocities, 1e-6)
    assert ok, r


# ---------------------------------------------------------------- edge cases
def test_empty_scene(cuda_lib):
    s = scenes.small_mixed()
    p = s.io_state.particles.subset(slice(0, 0))
    gpu = CudaState.from_io_state(IoState(0.0, p), s.consts)
    assert gpu.step(3, s.dt, s.gravity) == (0, 3)
    assert gpu.download().n == 0
    gpu.close()


def test_particles_leaving_domain_are_culled(cuda_lib, oracle_mod):
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    # shoot some particles out of the domain: strict bounds (cull_particles.rs:29-33)
    p.velocities[:50] = np.array([0.0, 0.0, -200.0], np.float32)
    io = IoState(0.0, p)
    consts = InputConsts(grid_node_size=s.consts.grid_node_size, domain_min=(0.0, 0.0, 0.29),
                         domain_max=(1.5, 1.5, 1.5))
    gpu = CudaState.from_io_state(io, consts)
    gpu.step(4, s.dt, s.gravity)
    out = gpu.download()
    ref = oracle_mod.OracleState(p, consts, None, fp64=True)
    ref.step(4, s.dt, s.gravity)
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    assert (out.flags & SV_TOMBSTONED).any()
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, dx=s.consts.grid_node_size)
    gpu.close()


def test_tombstoned_input_is_carried(cuda_lib):
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.flags[::3] |= SV_TOMBSTONED
    gpu = CudaState.from_io_state(IoState(0.0, p), s.consts)
    gpu.step(2, s.dt, s.gravity)
    out = gpu.download()
    dead = (p.flags & SV_TOMBSTONED) != 0
    np.testing.assert_array_equal(out.positions[dead], p.positions[dead])
    np.testing.assert_array_equal(out.position_gradients[dead], p.position_gradients[dead])
    gpu.close()


def test_inverted_particle_sets_failed_and_stops(cuda_lib):
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    # A compressive affine velocity field v = -k (x - c) on the first
    # (Neo-Hookean) box with k dt = 2: G2P recovers C = -k I and
    # F += dt C F flips F, so det F < 0 after one substep.
    box = np.arange(p.n) < p.n // 6
    c = p.positions[box].mean(0)
    k = 2.0 / s.dt
    p.velocities[:] = 0
    p.velocity_gradients[:] = 0
    p.position_gradients[:] = np.eye(3, dtype=np.float32).reshape(9)
    p.velocities[box] = -k * (p.positions[box] - c)
    p.velocity_gradients[box] = (-k * np.eye(3, dtype=np.float32)).reshape(9)
    gpu = CudaState.from_io_state(IoState(0.0, p), s.consts)
    status, done = gpu.step(5, s.dt, (0, 0, 0))
    assert status & SV_STATUS_PARTICLE_INVERTED
    assert done == 1
    out = gpu.download()
    assert (out.flags[box] & SV_FAILED).any()
    gpu.close()


def test_invalid_flags_rejected(cuda_lib):
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.flags[3] = 0  # neither solid nor fluid (initialization.rs:197-201)
    with pytest.raises(SvError):
        CudaState.from_io_state(IoState(0.0, p), s.consts)


def test_capacity_growth(cuda_lib, oracle_mod):
    s = scenes.small_mixed()
    small = CudaState.from_io_state(s.io_state, s.consts, Extras(block_capacity=4))
    big = CudaState.from_io_state(s.io_state, s.consts, Extras())
    assert small.step(3, s.dt, s.gravity) == (0, 3)
    big.step(3, s.dt, s.gravity)
    a, b = small.download(), big.download()
    compare_states(a, b, np.ones(a.n, bool), dx=s.consts.grid_node_size)
    small.close(), big.close()


def test_cancel_before_start(cuda_lib):
    from squishy_volumes_gb300 import Harness
    from squishy_volumes_gb300._abi import SV_STATUS_CANCELED

    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts)
    h = Harness()
    h.cancel()
    status, done = gpu.step(10, s.dt, s.gravity, h)
    assert status & SV_STATUS_CANCELED and done == 0
    gpu.close()


# ---------------------------------------------------------------- sand with mu = 0
def _sand_block(F0, mu=0.0, lam=0.0):
    from squishy_volumes_gb300 import Particles
    from squishy_volumes_gb300._abi import SV_USE_SAND_ALPHA

    dx = 0.05
    g = np.arange(8) * (dx / 2) + 0.4
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    n = len(pos)
    vol = np.full(n, (dx / 2) ** 3, np.float32)
    p = Particles(flags=np.full(n, SV_IS_SOLID | SV_USE_SAND_ALPHA, np.uint32), positions=pos,
                  position_gradients=np.tile(np.asarray(F0, np.float32).T.reshape(9), (n, 1)),
                  velocities=np.zeros((n, 3), np.float32), velocity_gradients=np.zeros((n, 9), np.float32),
                  mass=vol * 1000.0, initial_volume=vol, mu=np.full(n, mu, np.float32),
                  lambda_=np.full(n, lam, np.float32),
                  sand_alpha=np.full(n, scenes.friction_angle_to_alpha(np.deg2rad(30.0)), np.float32))
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
    return p, consts


def test_sand_with_zero_mu_projects_in_expansion(cuda_lib, oracle_mod):
    """(E, nu) = (0, 0.4), the last of the reference's test_lame_parameters
    (util/src/elastic.rs:679-689), gives mu = lambda = 0.  In expansion
    (e_tr >= 0) the reference sets F = U V^T whatever mu is
    (rust/crates/cpu/src/phase/advance_particles.rs:56-70), so a uniformly
    stretched block comes back to a rotation."""
    p, consts = _sand_block(np.diag([1.05, 1.02, 1.03]))
    gpu = CudaState.from_io_state(IoState(0.0, p), consts)
    assert gpu.step(2, 1e-4, (0.0, 0.0, 0.0)) == (0, 2)
    out = gpu.download()
    gpu.close()
    ref = oracle_mod.OracleState(p, consts, None, fp64=True)
    assert ref.step(2, 1e-4, (0.0, 0.0, 0.0)) == 0
    exp = ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    F = out.position_gradients.reshape(-1, 3, 3).astype(np.float64)
    # U V^T of a diagonal stretch is the identity
    assert np.abs(F - np.eye(3)).max() < 1e-5
    assert np.linalg.norm(out.position_gradients - exp.position_gradients) <= 1e-5 * np.linalg.norm(
        exp.position_gradients)


def test_sand_with_zero_mu_under_compression_is_the_references_assert(cuda_lib, oracle_mod):
    """Under compression with a deviatoric part (e_tr < 0, |e_hat| > 0) the
    reference asserts mu > 0 (advance_particles.rs:57) and its compute thread
    panics.  Here sv_step returns -1 with SV_STATUS_SAND_INVALID_MU in
    *status_out, and the oracle's step returns 3."""
    import ctypes as ct

    from squishy_volumes_gb300._abi import SV_STATUS_SAND_INVALID_MU, f32p, ptr

    p, consts = _sand_block(np.diag([0.95, 1.0, 1.02]))
    ref = oracle_mod.OracleState(p, consts, None, fp64=False)
    assert ref.step(1, 1e-4, (0.0, 0.0, 0.0)) == 3
    gpu = CudaState.from_io_state(IoState(0.0, p), consts)
    g = np.zeros(3, np.float32)
    status, done = ct.c_uint32(0), ct.c_uint32(0)
    rc = cuda_lib.sv_step(gpu._h, 3, ct.c_float(1e-4), ptr(g, f32p), None, ct.byref(status), ct.byref(done))
    assert rc == -1
    assert status.value & SV_STATUS_SAND_INVALID_MU
    assert b"mu <= 0" in cuda_lib.sv_last_error_string()
    assert done.value == 1  # the substep that met it completed; none after it ran
    # a stiff sand block (mu > 0) in the same state is projected, no error
    p2, consts2 = _sand_block(np.diag([0.95, 1.0, 1.02]), *scenes.lame(1e4, 0.3))
    gpu2 = CudaState.from_io_state(IoState(0.0, p2), consts2)
    assert gpu2.step(2, 1e-4, (0.0, 0.0, 0.0)) == (0, 2)
    gpu.close(), gpu2.close()
