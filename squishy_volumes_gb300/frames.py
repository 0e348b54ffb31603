"""Frame files and the frame cache, over the C ABI's sv_frame_* / sv_cache_*.

* ``write_frame`` / ``read_frame``: IoState::write / IoState::read
  (file_frame/src/io_state.rs:31-75) -- the reference's magic and version
  header, then bincode 1.3.3 over IoState.
* ``FrameCache``: the reference's StoreThread (cache/src/store_thread.rs:27-110)
  writing ``frame_%05d.bin`` files (cache/src/util.rs:9-11).  ``store`` queues
  the device-to-host copy of a CudaState's current state and returns; a
  writer thread in the library restores the particle order, serialises and
  writes.
"""

from __future__ import annotations

import ctypes as ct
import os
from typing import Optional

import numpy as np

from ._abi import SvFrame, check, f32p, i32p, load, ptr, u32p
from .state import CudaState, GridNodes, IoState, Particles

FRAME_VERSION = "0.3.4"  # the reference's file_util crate version (SV_FRAME_VERSION)

_PARTICLE_FIELDS = [  # (SvFrame field, Particles attribute, ctypes pointer, width, dtype)
    ("flags", "flags", u32p, 1, np.uint32),
    ("mass", "mass", f32p, 1, np.float32),
    ("initial_volume", "initial_volume", f32p, 1, np.float32),
    ("viscosity_dynamic", "viscosity_dynamic", f32p, 1, np.float32),
    ("viscosity_bulk", "viscosity_bulk", f32p, 1, np.float32),
    ("mu", "mu", f32p, 1, np.float32),
    ("lambda_", "lambda_", f32p, 1, np.float32),
    ("sand_alpha", "sand_alpha", f32p, 1, np.float32),
    ("exponent", "exponent", i32p, 1, np.int32),
    ("bulk_modulus", "bulk_modulus", f32p, 1, np.float32),
    ("elastic_energies", "elastic_energies", f32p, 1, np.float32),
    ("collider_bits", "collider_bits", u32p, 1, np.uint32),
    ("positions", "positions", f32p, 3, np.float32),
    ("position_gradients", "position_gradients", f32p, 9, np.float32),
    ("velocities", "velocities", f32p, 3, np.float32),
    ("velocity_gradients", "velocity_gradients", f32p, 9, np.float32),
    ("initial_positions", "initial_positions", f32p, 3, np.float32),
]
_GRID_FIELDS = [
    ("node_ids", "node_ids", i32p, 3, np.int32),
    ("node_collider_bits", "collider_bits", u32p, 1, np.uint32),
    ("node_masses", "masses", f32p, 1, np.float32),
    ("node_velocities", "velocities", f32p, 3, np.float32),
]


def _version(version: Optional[str]) -> Optional[bytes]:
    return None if version is None else version.encode()


def _struct(io: IoState, keep: list) -> SvFrame:
    """SvFrame pointing into io's arrays (kept alive through `keep`)."""
    p = io.particles
    f = SvFrame()
    f.time = float(io.time)
    f.n = p.n
    for name, attr, typ, _, dt in _PARTICLE_FIELDS:
        a = getattr(p, attr)
        if a is not None:
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
        setattr(f, name, ptr(a, typ))
    g = io.grid_nodes
    f.has_grid = 1 if g is not None else 0
    if g is not None:
        f.n_nodes = int(np.asarray(g.masses).shape[0])
        for name, attr, typ, _, dt in _GRID_FIELDS:
            a = np.ascontiguousarray(getattr(g, attr), dtype=dt)
            keep.append(a)
            setattr(f, name, ptr(a, typ))
    return f


def write_frame(path, io: IoState, version: Optional[str] = None) -> int:
    """Writes one frame file; returns its size in bytes."""
    keep: list = []
    f = _struct(io, keep)
    written = ct.c_uint64(0)
    check(load().sv_frame_write(os.fsencode(path), ct.byref(f), _version(version), ct.byref(written)))
    return int(written.value)


def read_frame(path, version: Optional[str] = None) -> IoState:
    """Reads one frame file (the version must match, like IoState::read)."""
    lib = load()
    head = SvFrame()
    check(lib.sv_frame_read(os.fsencode(path), _version(version), ct.byref(head)))
    n, m = int(head.n), int(head.n_nodes)
    f = SvFrame()
    f.n, f.n_nodes = n, m
    arrays = {}
    for name, _, typ, width, dt in _PARTICLE_FIELDS:
        a = np.zeros((n, width) if width > 1 else n, dtype=dt)
        arrays[name] = a
        setattr(f, name, ptr(a, typ))
    grid = {}
    if head.has_grid:
        for name, _, typ, width, dt in _GRID_FIELDS:
            a = np.zeros((m, width) if width > 1 else m, dtype=dt)
            grid[name] = a
            setattr(f, name, ptr(a, typ))
    check(lib.sv_frame_read(os.fsencode(path), _version(version), ct.byref(f)))
    particles = Particles(**{attr: arrays[name] for name, attr, _, _, _ in _PARTICLE_FIELDS})
    nodes = GridNodes(**{attr: grid[name] for name, attr, _, _, _ in _GRID_FIELDS}) if head.has_grid else None
    return IoState(float(f.time), particles, nodes)


class FrameCache:
    """The frame cache of one simulation: ``frame_%05d.bin`` files in
    ``directory``, numbered from ``first_frame``.  ``particles`` gives what
    the substep never changes (the parameters and the initial positions, in
    the original particle order); every stored frame repeats them."""

    def __init__(self, directory, particles: Particles, first_frame: int = 0, depth: int = 2,
                 version: Optional[str] = None):
        self._lib = load()
        self.directory = os.fspath(directory)
        statics = particles.copy()
        if statics.initial_positions is None:
            statics.initial_positions = statics.positions.copy()
        keep: list = []
        s = _struct(IoState(0.0, statics), keep)
        h = ct.c_void_p()
        check(self._lib.sv_cache_open(os.fsencode(self.directory), _version(version), ct.byref(s), int(first_frame),
                                      int(depth), ct.byref(h)))
        self._c = h

    def store(self, state: CudaState, store_grid: bool = False) -> None:
        """Queues the state's current frame (and the grid its last substep
        gathered); returns before the copy and the write finish."""
        check(self._lib.sv_cache_store(self._c, state._h, 1 if store_grid else 0))

    def store_io_state(self, io: IoState) -> None:
        """Queues a host frame (copied first), like StoreThread::store."""
        keep: list = []
        f = _struct(io, keep)
        check(self._lib.sv_cache_store_frame(self._c, ct.byref(f)))

    def check(self) -> None:
        """Raises once the writer thread has failed (StoreThread::check)."""
        check(self._lib.sv_cache_check(self._c))

    def flush(self) -> None:
        """Waits until every queued frame is on disk."""
        check(self._lib.sv_cache_flush(self._c))

    def info(self) -> tuple:
        """(frames written, bytes written)."""
        frames, nbytes = ct.c_uint64(0), ct.c_uint64(0)
        check(self._lib.sv_cache_info(self._c, ct.byref(frames), ct.byref(nbytes)))
        return int(frames.value), int(nbytes.value)

    def frame_path(self, frame: int) -> str:
        return os.path.join(self.directory, f"frame_{frame:05d}.bin")

    def close(self) -> None:
        if self._c:
            c, self._c = self._c, None
            check(self._lib.sv_cache_close(c))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
