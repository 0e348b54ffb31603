"""Host-side mirror of the reference's backend interface for the MPM substep.

The reference drives its CPU backend (rust/crates/cpu/src/cpu_state.rs) with
three calls, chosen behind `enum ComputeState`
(rust/crates/core/src/compute_thread.rs:101-117):

* ``CpuState::from_io_state(io_state)``            -> :meth:`CudaState.from_io_state`
* ``CpuState::produce_next_state(harness, frame_input, CpuRunParameters)``
                                                     -> :meth:`CudaState.produce_next_state`
* ``CpuState::to_io_state(store_grid)``              -> :meth:`CudaState.to_io_state`

The types below mirror ``IoState`` / ``Particles`` / ``GridNodes``
(rust/crates/file_frame/src/{io_state,particles,grid_nodes}.rs),
``InputConsts`` (rust/crates/file_input/src/header.rs:10-71) and the
cancellation half of ``Harness`` (rust/crates/xpu/src/harness.rs:53-144).
All compute goes through libsquishy_volumes_cuda.so; nothing here computes
physics.
"""

from __future__ import annotations

import ctypes as ct
import threading
from dataclasses import dataclass, field, fields
from typing import Optional

import numpy as np

from . import _abi
from ._abi import SvConsts, SvParticles, SvStats, check, f32p, i32p, ptr, u32p


# --------------------------------------------------------------------- types
@dataclass
class Particles:
    """file_frame::Particles (particles.rs:92-109) plus ParticleParameters
    (particles.rs:55-90) as per-particle arrays.  Matrices are [n, 9]
    column-major like nalgebra's Matrix3.  ``model`` .. ``plastic_j`` are
    additions (fixed-corotated and snow); ``model`` 0 means the reference's
    own Neo-Hookean / sand / fluid selection by flags."""

    flags: np.ndarray
    positions: np.ndarray
    position_gradients: np.ndarray
    velocities: np.ndarray
    velocity_gradients: np.ndarray
    mass: np.ndarray
    initial_volume: np.ndarray
    mu: Optional[np.ndarray] = None
    lambda_: Optional[np.ndarray] = None
    sand_alpha: Optional[np.ndarray] = None
    exponent: Optional[np.ndarray] = None
    bulk_modulus: Optional[np.ndarray] = None
    viscosity_dynamic: Optional[np.ndarray] = None
    viscosity_bulk: Optional[np.ndarray] = None
    elastic_energies: Optional[np.ndarray] = None
    collider_bits: Optional[np.ndarray] = None
    initial_positions: Optional[np.ndarray] = None
    model: Optional[np.ndarray] = None
    hardening: Optional[np.ndarray] = None
    crit_compression: Optional[np.ndarray] = None
    crit_stretch: Optional[np.ndarray] = None
    plastic_j: Optional[np.ndarray] = None

    _DTYPES = {
        "flags": np.uint32,
        "exponent": np.int32,
        "collider_bits": np.uint32,
        "model": np.uint32,
    }

    def __post_init__(self):
        for f in fields(self):
            v = getattr(self, f.name)
            if v is None:
                continue
            dt = self._DTYPES.get(f.name, np.float32)
            v = np.ascontiguousarray(v, dtype=dt)
            if f.name in ("positions", "velocities", "initial_positions"):
                v = v.reshape(-1, 3)
            elif f.name in ("position_gradients", "velocity_gradients"):
                v = v.reshape(-1, 9)
            setattr(self, f.name, v)

    @property
    def n(self) -> int:
        return int(self.flags.shape[0])

    def copy(self) -> "Particles":
        return Particles(**{f.name: (None if getattr(self, f.name) is None else getattr(self, f.name).copy())
                            for f in fields(self)})

    def subset(self, index) -> "Particles":
        return Particles(**{f.name: (None if getattr(self, f.name) is None else getattr(self, f.name)[index].copy())
                            for f in fields(self)})

    def nbytes(self) -> int:
        return sum(getattr(self, f.name).nbytes for f in fields(self) if getattr(self, f.name) is not None)

    def to_struct(self, keep=None) -> SvParticles:
        """SvParticles pointing into these arrays (they must stay alive)."""
        s = SvParticles()
        s.n = self.n
        s.flags = ptr(self.flags, u32p)
        s.positions = ptr(self.positions, f32p)
        s.position_gradients = ptr(self.position_gradients, f32p)
        s.velocities = ptr(self.velocities, f32p)
        s.velocity_gradients = ptr(self.velocity_gradients, f32p)
        s.elastic_energies = ptr(self.elastic_energies, f32p)
        s.collider_bits = ptr(self.collider_bits, u32p)
        s.mass = ptr(self.mass, f32p)
        s.initial_volume = ptr(self.initial_volume, f32p)
        s.viscosity_dynamic = ptr(self.viscosity_dynamic, f32p)
        s.viscosity_bulk = ptr(self.viscosity_bulk, f32p)
        s.mu = ptr(self.mu, f32p)
        s.lambda_ = ptr(self.lambda_, f32p)
        s.sand_alpha = ptr(self.sand_alpha, f32p)
        s.exponent = ptr(self.exponent, i32p)
        s.bulk_modulus = ptr(self.bulk_modulus, f32p)
        s.model = ptr(self.model, u32p)
        s.hardening = ptr(self.hardening, f32p)
        s.crit_compression = ptr(self.crit_compression, f32p)
        s.crit_stretch = ptr(self.crit_stretch, f32p)
        s.plastic_j = ptr(self.plastic_j, f32p)
        return s


@dataclass
class GridNodes:
    """file_frame::GridNodes (grid_nodes.rs:10-15); nodes with mass > 0."""

    node_ids: np.ndarray
    collider_bits: np.ndarray
    masses: np.ndarray
    velocities: np.ndarray


@dataclass
class IoState:
    """file_frame::IoState (io_state.rs:11-18)."""

    time: float
    particles: Particles
    grid_nodes: Optional[GridNodes] = None


@dataclass
class InputConsts:
    """The part of file_input::InputConsts (header.rs:10-71) the substep reads."""

    grid_node_size: float
    domain_min: tuple = (-100.0, -100.0, -100.0)
    domain_max: tuple = (100.0, 100.0, 100.0)
    simulation_scale: float = 1.0
    frames_per_second: int = 24

    def scaled_grid_node_size(self) -> float:
        return self.grid_node_size / self.simulation_scale

    def scaled_domain_min(self):
        return tuple(d / self.simulation_scale for d in self.domain_min)

    def scaled_domain_max(self):
        return tuple(d / self.simulation_scale for d in self.domain_max)

    def seconds_per_frame(self) -> float:
        return 1.0 / self.frames_per_second


@dataclass
class FrameData:
    """The inputs of frames a and b (xpu/src/frame_input.rs:33-65): gravity,
    particle goals and triangle-mesh colliders.  Arrays in the caller's
    particle order; b fields None means frame b = a (end of the input)."""

    frames_per_second: int
    frame: int
    gravity_a: tuple = (0.0, 0.0, -9.8)
    gravity_b: Optional[tuple] = None
    goal_flags_a: Optional[np.ndarray] = None      # [n] u32 (HAS_GOAL read)
    goal_flags_b: Optional[np.ndarray] = None
    goal_positions_a: Optional[np.ndarray] = None  # [n, 3]
    goal_positions_b: Optional[np.ndarray] = None
    triangles: Optional[np.ndarray] = None         # [t, 3] u32
    triangle_collider: Optional[np.ndarray] = None  # [t] u32 (0..15)
    vertex_positions_a: Optional[np.ndarray] = None  # [v, 3]
    vertex_positions_b: Optional[np.ndarray] = None
    friction_a: Optional[np.ndarray] = None        # [t]
    friction_b: Optional[np.ndarray] = None
    damping_a: Optional[np.ndarray] = None         # [t]
    damping_b: Optional[np.ndarray] = None
    leaf_size: float = 1.0

    @property
    def has_b(self) -> bool:
        return self.gravity_b is not None

    def to_struct(self, cls):
        """The C struct (sv_frame_input or the oracle's twin) and the arrays
        it points into (keep them alive while the struct is used)."""
        keep = {}

        def arr(name, dtype, shape_last=None):
            a = getattr(self, name)
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype)
            keep[name] = a
            return a

        s = cls()
        s.frames_per_second = int(self.frames_per_second)
        s.frame = int(self.frame)
        s.has_b = 1 if self.has_b else 0
        for k in range(3):
            s.gravity_a[k] = float(self.gravity_a[k])
            s.gravity_b[k] = float((self.gravity_b or self.gravity_a)[k])
        u32 = ct.POINTER(ct.c_uint32)
        f32 = ct.POINTER(ct.c_float)
        for name, dtype, typ in (("goal_flags_a", np.uint32, u32), ("goal_flags_b", np.uint32, u32),
                                 ("goal_positions_a", np.float32, f32), ("goal_positions_b", np.float32, f32),
                                 ("triangles", np.uint32, u32), ("triangle_collider", np.uint32, u32),
                                 ("vertex_positions_a", np.float32, f32), ("vertex_positions_b", np.float32, f32),
                                 ("friction_a", np.float32, f32), ("friction_b", np.float32, f32),
                                 ("damping_a", np.float32, f32), ("damping_b", np.float32, f32)):
            a = arr(name, dtype)
            setattr(s, name, a.ctypes.data_as(typ) if a is not None else ct.cast(None, typ))
        tri = keep.get("triangles")
        s.n_triangles = 0 if tri is None else tri.size // 3
        v = keep.get("vertex_positions_a")
        s.n_vertices = 0 if v is None else v.size // 3
        s.leaf_size = float(self.leaf_size)
        return s, keep


@dataclass
class Extras:
    """Options the reference does not have: a grid boundary plane, the
    int32-cell + fp32-offset position form, the fp64 SVD policy and the grid
    block capacity (0 = automatic)."""

    ground_mode: int = 0  # 0 off, 1 sticky, 2 slip
    ground_axis: int = 2
    ground_height: float = 0.0
    position_form: int = 0
    svd_fp64_policy: int = 1
    block_capacity: int = 0
    sort_interval: int = 0  # 0 adaptive, 1 every substep, k every k substeps
    host_transfer: int = 0  # 0 direct access to host arrays where possible, 1 staged copies
    deterministic_p2g: int = 0  # 1: P2G gathered per node in one fixed order (bit-reproducible)


@dataclass
class FrameInput:
    """The inputs of one frame the substep needs: the (interpolated) gravity
    (xpu/src/frame_input.rs, interpolate_input.rs:29)."""

    consts: InputConsts
    gravity: tuple = (0.0, 0.0, -9.8)


@dataclass
class RunParameters:
    """CpuRunParameters (cpu_state.rs:137-142)."""

    target_time: float
    max_time_step: float
    adaptive_time_steps: bool = False
    store_grid: bool = False


class Harness:
    """Cooperative cancellation (xpu/src/harness.rs:65-79)."""

    def __init__(self):
        self._flag = ct.c_int32(0)

    def cancel(self):
        self._flag.value = 1

    def canceled(self) -> bool:
        return bool(self._flag.value)


class EnergyError(RuntimeError):
    """A particle's position gradient got det <= 0 (util EnergyError::
    PositionGradientNonPositive); the state is still returned."""


class Canceled(RuntimeError):
    """The computation was canceled (cpu/src/errors.rs:11)."""


class ZeroTimeStep(RuntimeError):
    """The time step ended up being 0 (cpu/src/errors.rs:23)."""


# --------------------------------------------------------------------- backend
class CudaState:
    """GB300 backend with the reference CPU backend's call surface."""

    def __init__(self, handle: ct.c_void_p, n: int, time: float, consts: InputConsts, extras: Extras,
                 initial_positions: Optional[np.ndarray], template: Particles):
        self._lib = _abi.load()
        self._h = handle
        self.n = n
        self.consts = consts
        self.extras = extras
        self._initial_positions = initial_positions
        self._template = template
        self._frame_keep = None
        self.time = time
        direct = ct.c_uint32(0)
        check(self._lib.sv_set_host_transfer(self._h, int(extras.host_transfer), ct.byref(direct)))
        self._direct = bool(direct.value)  # downloads by kernels writing the host arrays

    # the simulation time lives in the handle (sv_step advances it)
    @property
    def time(self) -> float:
        t = ct.c_double(0.0)
        check(self._lib.sv_get_time(self._h, ct.byref(t)))
        return float(t.value)

    @time.setter
    def time(self, t: float):
        if float(t) != self.time:
            check(self._lib.sv_set_time(self._h, float(t)))

    def set_frame_input(self, frame: Optional["FrameData"]):
        """Loads the inputs of frames a and b (gravity, goals, colliders);
        None removes them.  See sv_set_frame_input in the C header."""
        if frame is None:
            check(self._lib.sv_set_frame_input(self._h, None))
            self._frame_keep = None
            return
        s, keep = frame.to_struct(_abi.SvFrameInput)
        check(self._lib.sv_set_frame_input(self._h, ct.byref(s)))
        self._frame_keep = keep

    # -- from_io_state (cpu_state.rs:25-66)
    @staticmethod
    def _consts(consts: InputConsts, extras: Extras) -> SvConsts:
        c = SvConsts()
        c.grid_node_size = consts.scaled_grid_node_size()
        for a in range(3):
            c.domain_min[a] = consts.scaled_domain_min()[a]
            c.domain_max[a] = consts.scaled_domain_max()[a]
        c.ground_mode = extras.ground_mode
        c.ground_axis = extras.ground_axis
        c.ground_height = extras.ground_height
        c.position_form = extras.position_form
        c.svd_fp64_policy = extras.svd_fp64_policy
        c.block_capacity = extras.block_capacity
        c.sort_interval = extras.sort_interval
        c.host_transfer = extras.host_transfer
        c.deterministic_p2g = extras.deterministic_p2g
        return c

    @classmethod
    def from_io_state(cls, io_state: IoState, consts: InputConsts, extras: Optional[Extras] = None) -> "CudaState":
        extras = extras or Extras()
        lib = _abi.load()
        c = cls._consts(consts, extras)
        p = io_state.particles
        s = p.to_struct()
        h = ct.c_void_p()
        check(lib.sv_create(ct.byref(c), ct.byref(s), ct.byref(h)))
        return cls(h, p.n, io_state.time, consts, extras, p.initial_positions, p)

    def close(self):
        if self._h:
            self._lib.sv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the substep loop
    def step(self, n_substeps: int, dt: float, gravity, harness: Optional[Harness] = None):
        """Runs n_substeps substeps; returns (status bits, substeps done)."""
        g = np.asarray(gravity, dtype=np.float32)
        status = ct.c_uint32(0)
        done = ct.c_uint32(0)
        cancel = ct.byref(harness._flag) if harness is not None else None
        check(self._lib.sv_step(self._h, int(n_substeps), float(dt), ptr(g, f32p), cancel, ct.byref(status),
                                ct.byref(done)))
        return int(status.value), int(done.value)

    def step_adaptive(self, target_time: float, max_time_step: float, gravity, harness: Optional[Harness] = None,
                      time: Optional[float] = None):
        """Adaptive substeps from `time` (default self.time) until target_time;
        returns (status bits, substeps done, time reached)."""
        g = np.asarray(gravity, dtype=np.float32)
        t = ct.c_double(self.time if time is None else time)
        status = ct.c_uint32(0)
        done = ct.c_uint32(0)
        cancel = ct.byref(harness._flag) if harness is not None else None
        rc = self._lib.sv_step_adaptive(self._h, ct.byref(t), float(target_time), float(max_time_step), ptr(g, f32p),
                                        cancel, ct.byref(status), ct.byref(done))
        if rc < 0:
            msg = self._lib.sv_last_error_string().decode()
            if "zero time step" in msg:
                raise ZeroTimeStep("The time step ended up being 0")
            check(rc)
        return int(status.value), int(done.value), float(t.value)

    def time_step_limits(self) -> dict:
        out = np.zeros(8, np.float32)
        check(self._lib.sv_time_step_limits(self._h, ptr(out, f32p)))
        keys = ("dt_force", "dt_scatter", "dt_advance", "velocity", "deformation", "sound", "isolated", "allowed")
        return {k: float(v) for k, v in zip(keys, out)}

    def produce_next_state(self, harness: Harness, frame_input: FrameInput, params: RunParameters):
        """cpu_state.rs:146-197: advance to target_time in substeps of
        max_time_step; returns (IoState, error-or-None) where the error is a
        buffered EnergyError (state still valid).  Canceled / ZeroTimeStep
        are raised, like the reference's outer Result."""
        if params.adaptive_time_steps:
            out, helper = self._download_ahead()
            try:
                status, done, t = self.step_adaptive(params.target_time, params.max_time_step, frame_input.gravity,
                                                     harness)
            finally:
                if helper is not None:
                    helper.join()
            error = None
            if status & _abi.SV_STATUS_PARTICLE_INVERTED:
                error = EnergyError("The position gradient has negative determinant")
            if status & _abi.SV_STATUS_CANCELED:
                raise Canceled("The computation was canceled")
            return self.to_io_state(params.store_grid, out), error
        dt = np.float32(params.max_time_step)
        if dt == 0:
            raise ZeroTimeStep("The time step ended up being 0")
        # the reference accumulates time in f64 one substep at a time; the
        # handle does the same (and does not count a failed substep)
        t = self.time
        n = 0
        while t < params.target_time:
            t += float(dt)
            n += 1
        out, helper = self._download_ahead()
        try:
            status, done = self.step(n, float(dt), frame_input.gravity, harness)
        finally:
            if helper is not None:
                helper.join()
        error = None
        if status & _abi.SV_STATUS_PARTICLE_INVERTED:
            error = EnergyError("The position gradient has negative determinant")
        if status & _abi.SV_STATUS_CANCELED:
            raise Canceled("The computation was canceled")
        return self.to_io_state(params.store_grid, out), error

    # -- to_io_state (cpu_state.rs:68-135)
    _DOWNLOADED = ("flags", "positions", "position_gradients", "velocities", "velocity_gradients",
                   "elastic_energies", "collider_bits", "plastic_j")

    def _new_download(self) -> Particles:
        """Particles with fresh arrays for what sv_download writes (every
        element of them) and the template's parameters."""
        t = self._template
        n = self.n
        return Particles(
            flags=np.empty(n, np.uint32),
            positions=np.empty((n, 3), np.float32),
            position_gradients=np.empty((n, 9), np.float32),
            velocities=np.empty((n, 3), np.float32),
            velocity_gradients=np.empty((n, 9), np.float32),
            mass=t.mass,
            initial_volume=t.initial_volume,
            mu=t.mu,
            lambda_=t.lambda_,
            sand_alpha=t.sand_alpha,
            exponent=t.exponent,
            bulk_modulus=t.bulk_modulus,
            viscosity_dynamic=t.viscosity_dynamic,
            viscosity_bulk=t.viscosity_bulk,
            elastic_energies=np.empty(n, np.float32),
            collider_bits=np.empty(n, np.uint32),
            initial_positions=self._initial_positions,
            model=t.model,
            hardening=t.hardening,
            crit_compression=t.crit_compression,
            crit_stretch=t.crit_stretch,
            plastic_j=np.empty(n, np.float32),
        )

    def _prepare(self, out: Particles) -> None:
        """Maps the pages of out's downloaded arrays (sv_prepare_host)."""
        arrays = [getattr(out, k) for k in self._DOWNLOADED]
        ptrs = (ct.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
        sizes = (ct.c_uint64 * len(arrays))(*[a.nbytes for a in arrays])
        check(self._lib.sv_prepare_host(ptrs, sizes, len(arrays)))

    def _download_ahead(self):
        """For the direct download: the frame's output arrays, and a thread
        that maps their pages while the substeps run (the calling thread
        only waits on the GPU then)."""
        if not self._direct:
            return None, None
        out = self._new_download()
        helper = threading.Thread(target=self._prepare, args=(out,), daemon=True)
        helper.start()
        return out, helper

    def download(self, out: Optional[Particles] = None) -> Particles:
        if out is None:
            out = self._new_download()
        s = out.to_struct()
        check(self._lib.sv_download(self._h, ct.byref(s)))
        return out

    def grid(self) -> GridNodes:
        cnt = ct.c_uint64(0)
        check(self._lib.sv_download_grid(self._h, None, None, None, 0, ct.byref(cnt)))
        m = int(cnt.value)
        ids = np.zeros((m, 3), np.int32)
        masses = np.zeros(m, np.float32)
        vel = np.zeros((m, 3), np.float32)
        check(self._lib.sv_download_grid(self._h, ptr(ids, i32p), ptr(masses, f32p), ptr(vel, f32p), m,
                                         ct.byref(cnt)))
        return GridNodes(ids, np.zeros(m, np.uint32), masses, vel)

    def to_io_state(self, store_grid: bool = False, out: Optional[Particles] = None) -> IoState:
        return IoState(self.time, self.download(out), self.grid() if store_grid else None)

    # -- inspection
    def p2g_only(self, dt: float, gravity) -> GridNodes:
        g = np.asarray(gravity, dtype=np.float32)
        check(self._lib.sv_p2g_only(self._h, float(dt), ptr(g, f32p)))
        return self.grid()

    def binning(self):
        n = self.n
        keys = np.zeros(n, np.uint32)
        perm = np.zeros(n, np.uint32)
        orig = np.zeros(n, np.uint32)
        check(self._lib.sv_binning(self._h, ptr(keys, u32p), ptr(perm, u32p), ptr(orig, u32p)))
        return keys, perm, orig

    def grid_layout(self):
        o = np.zeros(3, np.int32)
        nb = np.zeros(3, np.int32)
        check(self._lib.sv_grid_layout(self._h, ptr(o, i32p), ptr(nb, i32p)))
        return o, nb

    def stats(self) -> dict:
        s = SvStats()
        check(self._lib.sv_get_stats(self._h, ct.byref(s)))
        out = {}
        for name, typ in SvStats._fields_:
            v = getattr(s, name)
            out[name] = [float(x) for x in v] if hasattr(v, "__len__") else (float(v) if typ is ct.c_double else int(v))
        return out

    def set_stream(self, stream_handle: int):
        """Queue all work on a caller-owned cudaStream_t (0 = own stream)."""
        check(self._lib.sv_set_stream(self._h, ct.c_void_p(stream_handle or None)))

    # ---- learned closure of snow and sand (an addition; see sv_closure_* in the C header)
    def closure_harvest(self, dt: float, max_samples: int, augment: float = 0.0, seed: int = 0) -> int:
        total = ct.c_uint64(0)
        check(self._lib.sv_closure_harvest(self._h, float(dt), int(max_samples), float(augment), int(seed),
                                           ct.byref(total)))
        return int(total.value)

    def closure_harvest_from(self, other, dt: float, max_samples: int, augment: float = 0.0, seed: int = 0) -> int:
        """Harvest the current state of another state into this one's pool."""
        total = ct.c_uint64(0)
        check(self._lib.sv_closure_harvest_from(self._h, other._h, float(dt), int(max_samples), float(augment),
                                                int(seed), ct.byref(total)))
        return int(total.value)

    def closure_train(self, iterations: int, batch: int = 65536, lr: float = 3e-3, seed: int = 0) -> float:
        loss = ct.c_float(0.0)
        check(self._lib.sv_closure_train(self._h, int(iterations), int(batch), float(lr), int(seed), ct.byref(loss)))
        return float(loss.value)

    def closure_set_mode(self, mode: int):
        check(self._lib.sv_closure_set_mode(self._h, int(mode)))

    def closure_pool(self) -> dict:
        """Harvested pairs, and the yielding ones of the last training."""
        a, b = ct.c_uint64(0), ct.c_uint64(0)
        check(self._lib.sv_closure_pool(self._h, ct.byref(a), ct.byref(b)))
        return {"pairs": int(a.value), "yielding_pairs": int(b.value)}

    def closure_training_pool(self, first: int = 0, count: int = 0):
        """(X [count, 16], Y [count, 8], hull dict) of the normalised pool of
        the last training (count 0: all of it)."""
        from .closure import NIN, NOUT

        if count == 0:
            count = self.closure_pool()["yielding_pairs"] - first
        X = np.zeros((count, NIN), np.float32)
        Y = np.zeros((count, NOUT), np.float32)
        hull = np.zeros(80, np.float32)
        check(self._lib.sv_closure_get_pool(self._h, int(first), int(count), ptr(X, f32p), ptr(Y, f32p),
                                            ptr(hull, f32p)))
        keys = (("lo", 16), ("hi", 16), ("xm", 16), ("xs", 16), ("ym", 8), ("ys", 8))
        out, o = {}, 0
        for k, n in keys:
            out[k] = hull[o:o + n].copy()
            o += n
        return X, Y, out

    def closure_set_material_ranges(self, nu=(0.0, 0.0), friction_deg=(0.0, 0.0)):
        """Label training samples with Poisson's ratios / friction angles drawn
        from these ranges (all zero: the harvested materials)."""
        check(self._lib.sv_closure_set_material_ranges(self._h, float(nu[0]), float(nu[1]), float(friction_deg[0]),
                                                       float(friction_deg[1])))

    def closure_copy_from(self, other):
        """Take over the trained network, hull and normalisation of another state."""
        check(self._lib.sv_closure_copy(self._h, other._h))

    def closure_phase_times(self, dt: float) -> dict:
        out = (ct.c_double * 6)()
        check(self._lib.sv_closure_phase_times(self._h, float(dt), out))
        keys = ("plain_ms", "closed_form_ms", "network_all_ms", "particles", "yielding", "network_yielding_ms")
        return {k: float(v) for k, v in zip(keys, out)}

    def closure_evaluate(self, dt: float) -> dict:
        out = (ct.c_double * 12)()
        check(self._lib.sv_closure_evaluate(self._h, float(dt), out))
        keys = ("stress_err_learned", "stress_err_plain32", "f_err_learned", "f_err_plain32", "particles",
                "fallbacks", "stress_norm", "f_norm", "network", "residual_rejects", "stress_err_network_part",
                "stress_err_elastic_part")
        return {k: float(v) for k, v in zip(keys, out)}

    def closure_params(self) -> np.ndarray:
        from .closure import param_count

        p = np.zeros(param_count(), np.float32)
        check(self._lib.sv_closure_get_params(self._h, ptr(p, f32p)))
        return p

    def set_graphs(self, on: bool):
        check(self._lib.sv_set_graphs(self._h, 1 if on else 0))

    def set_host_transfer(self, mode: int) -> bool:
        """0: downloads by kernels writing the host arrays where the device
        can access pageable memory, 1: staged copies; returns whether the
        direct path is in use."""
        direct = ct.c_uint32(0)
        check(self._lib.sv_set_host_transfer(self._h, int(mode), ct.byref(direct)))
        return bool(direct.value)

    def autotune(self, dt: float, gravity, substeps_per_trial: int = 16):
        """Times the binning interval x CTAs-per-SM candidates on a snapshot
        of the state (restored afterwards) and keeps the fastest."""
        g = np.asarray(gravity, dtype=np.float32)
        si, cta = ct.c_uint32(0), ct.c_uint32(0)
        check(self._lib.sv_autotune(self._h, float(dt), ptr(g, f32p), int(substeps_per_trial), ct.byref(si),
                                    ct.byref(cta)))
        return {"sort_interval": int(si.value), "cta_per_sm": int(cta.value)}

    def set_profiling(self, on: bool):
        check(self._lib.sv_set_profiling(self._h, 1 if on else 0))

    def profile_report(self) -> str:
        buf = ct.create_string_buffer(1 << 16)
        check(self._lib.sv_profile_report(self._h, buf, len(buf)))
        return buf.value.decode()


def sort_pairs(keys: np.ndarray) -> np.ndarray:
    """Stable sorting permutation of u32 keys computed on the GPU."""
    keys = np.ascontiguousarray(keys, dtype=np.uint32)
    perm = np.zeros(keys.shape[0], np.uint32)
    check(_abi.load().sv_sort_pairs(ptr(keys, u32p), ptr(perm, u32p), keys.shape[0]))
    return perm


class BatchedCudaState(CudaState):
    """Many independent scenes in one handle (sv_create_batched): one set of
    launches advances them all.  Not in the reference, whose backend holds
    one scene; each scene keeps its own domain and cull bounds."""

    # what downloads take from the creating particles (the rest comes from
    # the device)
    _TEMPLATE_FIELDS = ("mass", "initial_volume", "mu", "lambda_", "sand_alpha", "exponent", "bulk_modulus",
                        "viscosity_dynamic", "viscosity_bulk", "model", "hardening", "crit_compression",
                        "crit_stretch", "initial_positions")

    def __init__(self, handle, counts, consts_list, extras, particles_list):
        total = sum(counts)
        # only the parameter arrays are merged: concatenating every state
        # array too cost about a quarter of a second for 7.5M particles
        merged = _concat_fields(particles_list, self._TEMPLATE_FIELDS)
        super().__init__(handle, total, 0.0, consts_list[0], extras, merged.initial_positions, merged)
        self.counts = list(counts)
        self.first = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.consts_list = list(consts_list)
        self._templates = list(particles_list)

    @classmethod
    def from_scenes(cls, io_states, consts_list, extras: Optional[Extras] = None) -> "BatchedCudaState":
        extras = extras or Extras()
        lib = _abi.load()
        k = len(io_states)
        cs = (SvConsts * k)(*[cls._consts(c, extras) for c in consts_list])
        keep = [s.particles for s in io_states]
        ps = (SvParticles * k)(*[p.to_struct() for p in keep])
        h = ct.c_void_p()
        check(lib.sv_create_batched(cs, ps, k, ct.byref(h)))
        return cls(h, [p.n for p in keep], consts_list, extras, keep)

    def scene_count(self) -> int:
        return int(self._lib.sv_scene_count(self._h))

    def download_scene(self, scene: int) -> Particles:
        t = self._templates[scene]
        m = t.n
        out = Particles(
            flags=np.zeros(m, np.uint32), positions=np.zeros((m, 3), np.float32),
            position_gradients=np.zeros((m, 9), np.float32), velocities=np.zeros((m, 3), np.float32),
            velocity_gradients=np.zeros((m, 9), np.float32), mass=t.mass, initial_volume=t.initial_volume,
            mu=t.mu, lambda_=t.lambda_, sand_alpha=t.sand_alpha, exponent=t.exponent, bulk_modulus=t.bulk_modulus,
            viscosity_dynamic=t.viscosity_dynamic, viscosity_bulk=t.viscosity_bulk,
            elastic_energies=np.zeros(m, np.float32), collider_bits=np.zeros(m, np.uint32),
            initial_positions=t.initial_positions, model=t.model, hardening=t.hardening,
            crit_compression=t.crit_compression, crit_stretch=t.crit_stretch, plastic_j=np.ones(m, np.float32))
        s = out.to_struct()
        check(self._lib.sv_download_scene(self._h, int(scene), ct.byref(s)))
        return out


def _concat_fields(parts, names):
    """The named fields of every part concatenated (None where any part has
    none), as attributes of a plain namespace."""
    from types import SimpleNamespace

    out = {}
    for name in names:
        vals = [getattr(p, name) for p in parts]
        out[name] = None if any(v is None for v in vals) else np.concatenate(vals)
    return SimpleNamespace(**out)
