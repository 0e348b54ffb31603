"""sv_create's host pass over the particles (no GPU needed: it rejects invalid
input before any device call).  Bodies are runs of identical parameters; the
pass reuses the previous particle's material across such a run, so these
cases put the invalid particle inside runs and across the host threads'
parts, and check that the lowest invalid particle is the one reported, as a
sequential pass over the reference's initialization
(core/src/initialization.rs:197-201, util/src/elastic.rs:527-543) would."""

from dataclasses import fields

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, IoState, Particles, scenes
from squishy_volumes_gb300._abi import SvError


def _tiled(p: Particles, reps: int) -> Particles:
    """reps copies of p, one after another (runs of identical parameters)."""
    kw = {}
    for f in fields(p):
        v = getattr(p, f.name)
        kw[f.name] = None if v is None else np.concatenate([v] * reps)
    return Particles(**kw)


def _create_error(p: Particles, consts) -> str:
    with pytest.raises(SvError) as e:
        CudaState.from_io_state(IoState(0.0, p), consts).close()
    return str(e.value)


def test_invalid_flags_inside_a_run():
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.flags[500:520] = 0
    assert "particle 500: exactly one of IS_SOLID and IS_FLUID" in _create_error(p, s.consts)


def test_invalid_fluid_exponent_after_identical_fluid_particles():
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    fluid = np.flatnonzero(p.flags & 2)  # IS_FLUID
    k = int(fluid[len(fluid) // 2])
    p.exponent[k] = 1
    assert f"particle {k}: exponent must be greater than 1" in _create_error(p, s.consts)


def test_lowest_invalid_particle_across_thread_parts():
    s = scenes.small_mixed()
    base = s.io_state.particles
    p = _tiled(base, 400)  # 360k particles: several host threads' parts
    n = p.flags.shape[0]
    assert n > 4 * (1 << 16)
    hi, lo = n - 1000, n // 2 + 17
    p.flags[hi] = 0
    p.flags[lo] = 3  # both IS_SOLID and IS_FLUID
    assert f"particle {lo}: exactly one of IS_SOLID and IS_FLUID" in _create_error(p, s.consts)


def test_non_finite_position_is_reported_after_parameters():
    s = scenes.small_mixed()
    p = s.io_state.particles.copy()
    p.positions[700, 1] = np.nan
    assert "non-finite particle position" in _create_error(p, s.consts)
    p.flags[800] = 0  # a parameter error anywhere comes first
    assert "particle 800:" in _create_error(p, s.consts)
