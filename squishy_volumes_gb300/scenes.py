"""Seeded synthetic scenes with the shapes, sizes and materials of the
benchmark configurations (no recorded scene data is used).

Particles are sampled like the reference's Blender input: each particle
stands for a cube of side ``size`` (here half a grid cell, i.e. two particles
per cell axis), so ``initial_volume = size**3`` and ``mass = density *
initial_volume`` (rust/crates/core/src/initialization.rs:202-205), with
Lamé parameters from Young's modulus and Poisson's ratio (util/src/
elastic.rs:52-64).  Positions are jittered uniformly within each sub-cell.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from ._abi import SV_IS_FLUID, SV_IS_SOLID, SV_MODEL_FIXED_COROTATED, SV_MODEL_REFERENCE, SV_MODEL_SNOW, SV_USE_SAND_ALPHA
from .state import Extras, InputConsts, IoState, Particles


def lame(youngs_modulus: float, poissons_ratio: float):
    """mu and lambda from E and nu (util/src/elastic.rs:52-64)."""
    mu = youngs_modulus / 2.0 / (1.0 + poissons_ratio)
    la = youngs_modulus * poissons_ratio / (1.0 + poissons_ratio) / (1.0 - 2.0 * poissons_ratio)
    return mu, la


def friction_angle_to_alpha(phi_rad: float) -> float:
    """Drucker-Prager cone coefficient from a friction angle (Klar et al.
    2016); the reference takes "Sand Alpha" as a raw input instead."""
    s = math.sin(phi_rad)
    return math.sqrt(2.0 / 3.0) * 2.0 * s / (3.0 - s)


@dataclass
class Material:
    kind: str  # "neo_hookean", "fixed_corotated", "snow", "sand", "fluid"
    density: float = 1000.0
    youngs_modulus: float = 1e5
    poissons_ratio: float = 0.3
    friction_angle_deg: float = 35.0
    crit_compression: float = 2.5e-2
    crit_stretch: float = 7.5e-3
    hardening: float = 10.0
    bulk_modulus: float = 1e5
    exponent: int = 7


@dataclass
class Scene:
    name: str
    io_state: IoState
    consts: InputConsts
    extras: Extras
    dt: float
    substeps: int
    gravity: tuple = (0.0, 0.0, -9.81)
    meta: dict = field(default_factory=dict)


def jittered_box(rng, lo, dims, spacing):
    """dims[0] x dims[1] x dims[2] particles, one per sub-cell of size
    `spacing`, jittered uniformly inside it; lo is the box's min corner."""
    ii, jj, kk = np.meshgrid(np.arange(dims[0]), np.arange(dims[1]), np.arange(dims[2]), indexing="ij")
    idx = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64)
    jitter = rng.random(idx.shape)
    return (np.asarray(lo, np.float64) + (idx + jitter) * spacing).astype(np.float32)


def build_particles(blocks) -> Particles:
    """blocks: list of (positions [m,3], Material, velocity [3] or [m,3], size)."""
    parts = []
    for pos, mat, vel, size in blocks:
        m = pos.shape[0]
        v0 = np.float32(size) ** 3
        rec = {
            "flags": np.full(m, SV_IS_FLUID if mat.kind == "fluid" else SV_IS_SOLID, np.uint32),
            "positions": pos,
            "position_gradients": np.tile(np.eye(3, dtype=np.float32).reshape(1, 9), (m, 1)),
            "velocities": np.broadcast_to(np.asarray(vel, np.float32), (m, 3)).copy(),
            "velocity_gradients": np.zeros((m, 9), np.float32),
            "mass": np.full(m, v0 * np.float32(mat.density), np.float32),
            "initial_volume": np.full(m, v0, np.float32),
            "mu": np.zeros(m, np.float32),
            "lambda_": np.zeros(m, np.float32),
            "sand_alpha": np.zeros(m, np.float32),
            "exponent": np.zeros(m, np.int32),
            "bulk_modulus": np.zeros(m, np.float32),
            "model": np.full(m, SV_MODEL_REFERENCE, np.uint32),
            "hardening": np.zeros(m, np.float32),
            "crit_compression": np.zeros(m, np.float32),
            "crit_stretch": np.zeros(m, np.float32),
            "plastic_j": np.ones(m, np.float32),
            "elastic_energies": np.zeros(m, np.float32),
            "collider_bits": np.zeros(m, np.uint32),
        }
        if mat.kind == "fluid":
            rec["exponent"][:] = mat.exponent
            rec["bulk_modulus"][:] = mat.bulk_modulus
        else:
            mu, la = lame(mat.youngs_modulus, mat.poissons_ratio)
            rec["mu"][:] = mu
            rec["lambda_"][:] = la
            if mat.kind == "sand":
                rec["flags"] |= SV_USE_SAND_ALPHA
                rec["sand_alpha"][:] = friction_angle_to_alpha(math.radians(mat.friction_angle_deg))
            elif mat.kind == "fixed_corotated":
                rec["model"][:] = SV_MODEL_FIXED_COROTATED
            elif mat.kind == "snow":
                rec["model"][:] = SV_MODEL_SNOW
                rec["hardening"][:] = mat.hardening
                rec["crit_compression"][:] = mat.crit_compression
                rec["crit_stretch"][:] = mat.crit_stretch
        parts.append(rec)
    keys = parts[0].keys()
    merged = {k: np.concatenate([p[k] for p in parts]) for k in keys}
    merged["initial_positions"] = merged["positions"].copy()
    return Particles(**merged)


def cube_64k(seed: int = 1) -> Scene:
    """Plain MLS-MPM, unit-cube domain, dx = 1/128, one fixed-corotated cube of
    40^3 = 64,000 particles (2 per cell axis, jittered), E = 1e5, nu = 0.3,
    density 1000, v = 0, gravity -9.81, dt = 1e-4, 100 substeps, sticky
    ground plane."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / 128
    mat = Material("fixed_corotated", youngs_modulus=1e5, poissons_ratio=0.3)
    pos = jittered_box(rng, (54 * dx, 54 * dx, 20 * dx), (40, 40, 40), dx / 2)
    p = build_particles([(pos, mat, (0, 0, 0), dx / 2)])
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
    extras = Extras(ground_mode=1, ground_axis=2, ground_height=4 * dx)
    return Scene("cube_64k", IoState(0.0, p), consts, extras, dt=1e-4, substeps=100)


def three_boxes_1m(seed: int = 2, per_box_dims=(69, 69, 70)) -> Scene:
    """Plain method, ~1M particles on a sparse 4^3-block grid over a 256^3
    domain (dx = 1/256): three seeded jittered boxes of ~333k particles --
    fixed-corotated (E = 2e5, nu = 0.3), snow (E = 1.4e5, nu = 0.2,
    theta_c = 2.5e-2, theta_s = 7.5e-3, xi = 10) and Drucker-Prager sand
    (E = 3.5e5, nu = 0.3, friction angle 35 deg).  Each box gets one velocity
    drawn uniformly from [-1, 1]^3 m/s.  dt = 5e-5, 500 substeps, sticky
    ground plane."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / 256
    mats = [
        Material("fixed_corotated", youngs_modulus=2e5, poissons_ratio=0.3),
        Material("snow", youngs_modulus=1.4e5, poissons_ratio=0.2, crit_compression=2.5e-2,
                 crit_stretch=7.5e-3, hardening=10.0),
        Material("sand", youngs_modulus=3.5e5, poissons_ratio=0.3, friction_angle_deg=35.0),
    ]
    corners = [(40, 40, 60), (110, 130, 90), (180, 60, 120)]
    blocks = []
    for mat, lo in zip(mats, corners):
        pos = jittered_box(rng, tuple(c * dx for c in lo), per_box_dims, dx / 2)
        vel = rng.uniform(-1.0, 1.0, 3)
        blocks.append((pos, mat, vel, dx / 2))
    p = build_particles(blocks)
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
    extras = Extras(ground_mode=1, ground_axis=2, ground_height=8 * dx)
    return Scene("three_boxes_1m", IoState(0.0, p), consts, extras, dt=5e-5, substeps=500)


def dam_break_8m(seed: int = 3, fluid_dims=(410, 366, 40), box_dims=(80, 80, 78), position_form: int = 1) -> Scene:
    """Precision form, ~8M particles, sparse grid over a 512^3 domain
    (dx = 1/512): a weakly compressible fluid column (bulk modulus 1e5,
    exponent 7, ~6M particles, 40 % of the domain width) plus four
    Neo-Hookean boxes (E = 1e5, nu = 0.35, ~2M particles).  Positions are an
    int32 cell index + fp32 offset.  dt = 2e-5, 200 substeps."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / 512
    fluid = Material("fluid", bulk_modulus=1e5, exponent=7)
    elastic = Material("neo_hookean", youngs_modulus=1e5, poissons_ratio=0.35)
    blocks = [(jittered_box(rng, (10 * dx, 10 * dx, 10 * dx), fluid_dims, dx / 2), fluid, (0, 0, 0), dx / 2)]
    for lo in [(260, 40, 20), (360, 40, 20), (260, 200, 20), (360, 200, 20)]:
        blocks.append((jittered_box(rng, tuple(c * dx for c in lo), box_dims, dx / 2), elastic, (0, 0, 0), dx / 2))
    p = build_particles(blocks)
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
    extras = Extras(ground_mode=1, ground_axis=2, ground_height=4 * dx, position_form=position_form)
    return Scene("dam_break_8m", IoState(0.0, p), consts, extras, dt=2e-5, substeps=200)


def small_mixed(n_per_material: int = 300, seed: int = 5, dx: float = 0.05, deform: float = 0.05,
                speed: float = 0.5) -> Scene:
    """A small scene for parity tests: one jittered box per material kind
    (Neo-Hookean, sand, fluid, fixed-corotated, snow, Neo-Hookean with
    viscosity) with random velocities, velocity gradients and deformed F."""
    rng = np.random.default_rng(seed)
    kinds = ["neo_hookean", "sand", "fluid", "fixed_corotated", "snow", "viscous"]
    side = max(2, round(n_per_material ** (1 / 3)))
    blocks = []
    for i, kind in enumerate(kinds):
        mk = "neo_hookean" if kind == "viscous" else kind
        mat = Material(mk, youngs_modulus=1e4 * (1 + i), poissons_ratio=0.3, bulk_modulus=1e3, exponent=7)
        lo = (0.2 + 0.6 * (i % 3) / 3, 0.2 + 0.3 * (i // 3), 0.3)
        pos = jittered_box(rng, lo, (side, side, side), dx / 2)
        blocks.append((pos, mat, (0, 0, 0), dx / 2))
    p = build_particles(blocks)
    n = p.n
    p.velocities[:] = rng.uniform(-speed, speed, (n, 3)).astype(np.float32)
    p.velocity_gradients[:] = rng.uniform(-1.0, 1.0, (n, 9)).astype(np.float32)
    F = np.eye(3, dtype=np.float64)[None] + deform * rng.uniform(-1, 1, (n, 3, 3))
    p.position_gradients[:] = F.transpose(0, 2, 1).reshape(n, 9).astype(np.float32)  # column-major
    visc = np.arange(n) >= 5 * side ** 3
    from ._abi import SV_USE_VISCOSITY

    p.flags[visc] |= SV_USE_VISCOSITY
    p.viscosity_dynamic = np.where(visc, 0.5, 0.0).astype(np.float32)
    p.viscosity_bulk = np.where(visc, 0.25, 0.0).astype(np.float32)
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.5, 1.5, 1.5))
    return Scene("small_mixed", IoState(0.0, p), consts, Extras(), dt=1e-4, substeps=10)





def batched_64(seed: int = 4, n_scenes: int = 64, median: float = 8e4, sigma: float = 1.0,
               lo: int = 10_000, hi: int = 500_000):
    """Batched form: independent scenes, each a seeded jittered box of one
    material drawn from {fixed-corotated elastic, snow, sand} on its own
    256^3 grid over the unit cube (dx = 1/256).  Particle counts are
    lognormal, clipped to [10k, 500k]; E ~ U[5e4, 5e5], nu ~ U[0.2, 0.4],
    friction angle ~ U[25, 40] deg; dt = 5e-5, 300 substeps, sticky ground."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / 256
    counts = np.clip(np.exp(rng.normal(math.log(median), sigma, n_scenes)), lo, hi).astype(np.int64)
    scenes_out = []
    for s, cnt in enumerate(counts):
        kind = ["fixed_corotated", "snow", "sand"][int(rng.integers(0, 3))]
        E, nu = float(rng.uniform(5e4, 5e5)), float(rng.uniform(0.2, 0.4))
        phi = float(rng.uniform(25.0, 40.0))
        mat = Material(kind, youngs_modulus=E, poissons_ratio=nu, friction_angle_deg=phi)
        side = max(2, int(round(cnt ** (1 / 3))))
        dims = (side, side, max(2, int(round(cnt / side / side))))
        lo_c = rng.integers(20, 256 - 20 - dims[0] // 2, 2)
        pos = jittered_box(rng, (lo_c[0] * dx, lo_c[1] * dx, 30 * dx), dims, dx / 2)
        p = build_particles([(pos, mat, rng.uniform(-0.5, 0.5, 3), dx / 2)])
        consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
        extras = Extras(ground_mode=1, ground_axis=2, ground_height=8 * dx, position_form=1)
        scenes_out.append(Scene(f"batched_{s}", IoState(0.0, p), consts, extras, dt=5e-5, substeps=300,
                                meta={"material": kind, "E": E, "nu": nu, "friction_deg": phi}))
    return scenes_out


def snow_sand_2m(seed: int = 6, box_dims=(100, 100, 100), dx: float = 1.0 / 512) -> Scene:
    """Learned-closure workload: a snow box (E = 1.4e5, nu = 0.2,
    theta_c = 2.5e-2, theta_s = 7.5e-3, xi = 10) and a Drucker-Prager sand
    box (E = 3.5e5, nu = 0.3, friction angle 35 deg) of ~1M particles each
    (2 per cell axis, jittered), moving towards each other at 1 m/s each
    (2 m/s closing speed) over a 512^3 domain (dx = 1/512).  dt = 5e-5,
    1000 substeps, sticky ground plane, cell + offset positions."""
    rng = np.random.default_rng(seed)
    snow = Material("snow", youngs_modulus=1.4e5, poissons_ratio=0.2, crit_compression=2.5e-2, crit_stretch=7.5e-3,
                    hardening=10.0)
    sand = Material("sand", youngs_modulus=3.5e5, poissons_ratio=0.3, friction_angle_deg=35.0)
    cells = int(round(1.0 / dx))
    side = box_dims[0] // 2  # cells per box edge
    gap = max(4, side // 10)
    x0, y0, z0 = cells // 2 - side - gap // 2, (2 * cells) // 5, 16
    blocks = [
        (jittered_box(rng, (x0 * dx, y0 * dx, z0 * dx), box_dims, dx / 2), snow, (1.0, 0.0, 0.0), dx / 2),
        (jittered_box(rng, ((x0 + side + gap) * dx, y0 * dx, z0 * dx), box_dims, dx / 2), sand, (-1.0, 0.0, 0.0),
         dx / 2),
    ]
    p = build_particles(blocks)
    consts = InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0))
    extras = Extras(ground_mode=1, ground_axis=2, ground_height=8 * dx, position_form=1)
    return Scene("snow_sand_2m", IoState(0.0, p), consts, extras, dt=5e-5, substeps=1000)


def dam_break_1m(seed: int = 3) -> Scene:
    """dam_break_8m at one eighth of the particles (half the extent per axis
    of the fluid column and the boxes; same dx, materials and time step): a
    case of the same kernels small enough for a full profiler capture."""
    s = dam_break_8m(seed, fluid_dims=(205, 183, 20), box_dims=(40, 40, 39))
    s.name = "dam_break_1m"
    return s


SCENES = {
    "cube_64k": cube_64k,
    "three_boxes_1m": three_boxes_1m,
    "dam_break_8m": dam_break_8m,
    "dam_break_1m": dam_break_1m,
    "small_mixed": small_mixed,
    "batched_64": batched_64,
    "snow_sand_2m": snow_sand_2m,
}
