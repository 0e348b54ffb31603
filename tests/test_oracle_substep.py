"""The CPU oracle's whole substep (CPU only): conservation laws of the
transfer, exact invariants, precision-twin agreement, the committed golden
vectors, and the binning-key contract shared with the CUDA library."""

from pathlib import Path

import numpy as np
import pytest

import oracle
from squishy_volumes_gb300 import Extras, InputConsts, IoState, Particles, scenes
from squishy_volumes_gb300._abi import SV_TOMBSTONED

GOLDEN = Path(__file__).parent / "golden" / "oracle_small_mixed.npz"


def golden_particles(g):
    names = ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "mass",
             "initial_volume", "mu", "lambda_", "sand_alpha", "exponent", "bulk_modulus", "viscosity_dynamic",
             "viscosity_bulk", "model", "hardening", "crit_compression", "crit_stretch", "plastic_j"]
    return Particles(**{k: g[f"in_{k}"] for k in names})


def golden_consts(g):
    return InputConsts(grid_node_size=float(g["grid_node_size"]), domain_min=tuple(g["domain_min"]),
                       domain_max=tuple(g["domain_max"]))


def test_golden_vectors_reproduce():
    g = np.load(GOLDEN)
    p = golden_particles(g)
    o = oracle.OracleState(p, golden_consts(g), None, fp64=True, threads=2)
    assert o.step(int(g["substeps"]), float(g["dt"]), g["gravity"]) == 0
    out = o.download()
    np.testing.assert_array_equal(out.flags, g["out_flags"])
    for k in ["positions", "position_gradients", "velocities", "velocity_gradients", "elastic_energies", "plastic_j"]:
        np.testing.assert_allclose(getattr(out, k), g[f"out_{k}"], rtol=1e-5, atol=1e-7, err_msg=k)


def test_p2g_conserves_mass_and_momentum():
    s = scenes.small_mixed()
    p = s.io_state.particles
    o = oracle.OracleState(p, s.consts, None, fp64=True)
    o.p2g_only(s.dt, s.gravity)
    ids, m, v = o.grid()
    np.testing.assert_allclose(m.sum(dtype=np.float64), p.mass.sum(dtype=np.float64), rtol=1e-6)
    grid_mom = (m[:, None].astype(np.float64) * v).sum(0)
    part_mom = (p.mass[:, None].astype(np.float64) * (p.velocities + s.dt * np.asarray(s.gravity))).sum(0)
    scale = (p.mass[:, None] * np.abs(p.velocities)).sum()
    assert np.all(np.abs(grid_mom - part_mom) < 1e-5 * scale)


def test_rigid_translation_is_exact():
    """Uniform velocity, F = I, C = 0, no gravity: the transfer reproduces the
    velocity, C stays 0 and x moves by v dt."""
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.velocities[:] = np.array([0.3, -0.2, 0.1], np.float32)
    p.velocity_gradients[:] = 0
    p.position_gradients[:] = np.eye(3, dtype=np.float32).reshape(9)
    p.flags &= ~np.uint32(4)  # no viscosity
    o = oracle.OracleState(p, s.consts, None, fp64=True)
    assert o.step(1, s.dt, (0, 0, 0)) == 0
    out = o.download()
    np.testing.assert_allclose(out.velocities, p.velocities, atol=1e-6)
    np.testing.assert_allclose(out.velocity_gradients, 0, atol=1e-4)
    np.testing.assert_allclose(out.positions, p.positions + s.dt * p.velocities, atol=1e-7)


def test_fp32_and_fp64_twins_agree():
    s = scenes.small_mixed()
    a = oracle.OracleState(s.io_state.particles, s.consts, None, fp64=False)
    b = oracle.OracleState(s.io_state.particles, s.consts, None, fp64=True)
    a.step(s.substeps, s.dt, s.gravity)
    b.step(s.substeps, s.dt, s.gravity)
    x, y = a.download(), b.download()
    live = (y.flags & SV_TOMBSTONED) == 0
    for k, tol in [("positions", 1e-6), ("velocities", 1e-4), ("position_gradients", 1e-5)]:
        d = np.linalg.norm(getattr(x, k)[live].astype(np.float64) - getattr(y, k)[live])
        assert d <= tol * np.linalg.norm(getattr(y, k)[live]), k


def test_cull_is_strict():
    """cull_particles.rs:29-33: a particle exactly on the domain bound is culled."""
    s = scenes.small_mixed()
    p = s.io_state.particles.subset(slice(0, 8)).copy()
    p.velocities[:] = 0
    p.velocity_gradients[:] = 0
    lo = float(p.positions[:, 0].min())
    consts = InputConsts(grid_node_size=s.consts.grid_node_size, domain_min=(lo, -10.0, -10.0),
                         domain_max=(10.0, 10.0, 10.0))
    o = oracle.OracleState(p, consts, None, fp64=True)
    o.step(1, 1e-9, (0, 0, 0))
    out = o.download()
    on_bound = p.positions[:, 0] == lo
    assert on_bound.any()
    assert np.all((out.flags[on_bound] & SV_TOMBSTONED) != 0)


def test_binning_keys_contract_and_stable_sort():
    rng = np.random.default_rng(4)
    n = 5000
    pos = rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32)
    flags = np.ones(n, np.uint32)
    flags[::13] |= SV_TOMBSTONED
    dx = 1.0 / 64
    origin = np.array([-5, -5, -5], np.int32)
    nb = np.array([20, 20, 20], np.int32)
    keys = oracle.binning_keys(pos, flags, dx, origin, nb)
    c = np.floor(pos / np.float32(dx) - np.float32(0.5)).astype(np.int64) - origin
    exp = ((((c[:, 0] >> 2) * nb[1] + (c[:, 1] >> 2)) * nb[2] + (c[:, 2] >> 2)) << 6) | (
        (c[:, 0] & 3) << 4 | (c[:, 1] & 3) << 2 | (c[:, 2] & 3))
    exp = exp.astype(np.uint32)
    exp[(flags & SV_TOMBSTONED) != 0] = 0xFFFFFFFF
    np.testing.assert_array_equal(keys, exp)
    np.testing.assert_array_equal(oracle.stable_sort_perm(keys), np.argsort(keys, kind="stable"))


def test_energy_error_stops_and_flags():
    """A particle that inverts gets FAILED and the oracle reports the energy
    error (advance_particles.rs:73-74, cpu_state.rs:178-183)."""
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    box = np.arange(p.n) < p.n // 6
    c = p.positions[box].mean(0)
    k = 2.0 / s.dt
    p.velocities[:] = 0
    p.velocity_gradients[:] = 0
    p.position_gradients[:] = np.eye(3, dtype=np.float32).reshape(9)
    p.velocities[box] = -k * (p.positions[box] - c)
    p.velocity_gradients[box] = (-k * np.eye(3, dtype=np.float32)).reshape(9)
    o = oracle.OracleState(p, s.consts, None, fp64=True)
    assert o.step(3, s.dt, (0, 0, 0)) == 1
    out = o.download()
    assert (out.flags[box] & 64).any()
