"""CPU checker for the frame files (test infrastructure only).

A restatement, in plain Python, of what the reference writes into a cache
frame: IoState::write (rust/crates/file_frame/src/io_state.rs:31-64) puts the
32 magic bytes (io_state.rs:20-29) and the 64 version bytes
(rust/crates/file_util/src/lib.rs:27-70, the crate version zero padded), then
``bincode::serialize_into`` of IoState.  bincode is the crates.io dependency
bincode 1.3.3 (rust/Cargo.toml:14, rust/Cargo.lock), not vendored in the
reference; its published format for the serde data model with the options of
its top-level functions is restated here:

* integers and floats little endian, fixed width;
* a struct is its fields in declaration order, [T; N] is N values of T;
* Vec<T> is its length as u64, then the elements;
* Option<T> is u8 0 (None) or u8 1 followed by the value;
* an enum is its variant index as u32, then the variant's fields;
* a newtype struct (ParticleFlags(u32)) is its field.

The types, in order: IoState { time: f64, particles: Particles, grid_nodes:
Option<GridNodes> } (io_state.rs:11-18); Particles { flags, parameters,
elastic_energies, collider_bits, positions, position_gradients, velocities,
velocity_gradients, initial_positions } (file_frame/src/particles.rs:92-109);
ParticleParameters { mass, initial_volume, viscosity: Option<{dynamic,
bulk}>, specific: Solid { mu, lambda, sand_alpha: Option<f32> } | Fluid {
exponent: i32, bulk_modulus } } (particles.rs:55-90); GridNodes { node_ids:
Vec<[i32; 3]>, collider_bits: Vec<u32>, masses: Vec<f32>, velocites:
Vec<[f32; 3]> } (grid_nodes.rs:10-15).

The encoder works value by value with ``struct``, independently of the
library's writer, so a byte-for-byte comparison checks the writer.
"""

from __future__ import annotations

import struct

import numpy as np

MAGIC = b"Squishy Volumes Frame File Magic"
VERSION_LEN = 64
IS_FLUID, USE_VISCOSITY, USE_SAND_ALPHA = 1 << 1, 1 << 2, 1 << 3


def header(version: str) -> bytes:
    v = version.encode()
    assert len(v) <= VERSION_LEN
    return MAGIC + v + bytes(VERSION_LEN - len(v))


def _vec(values, fmt: str) -> bytes:
    """Vec<T> of scalars (fmt one struct code) or of fixed arrays."""
    flat = list(np.asarray(values).reshape(len(values), -1)) if len(values) else []
    out = [struct.pack("<Q", len(values))]
    for row in flat:
        for x in row:
            out.append(struct.pack("<" + fmt, x.item()))
    return b"".join(out)


def encode(time, p: dict, grid: dict | None, version: str) -> bytes:
    """Bytes of a frame file.  p: flags, mass, initial_volume,
    viscosity_dynamic, viscosity_bulk, mu, lambda_, sand_alpha, exponent,
    bulk_modulus, elastic_energies, collider_bits, positions,
    position_gradients, velocities, velocity_gradients, initial_positions
    (numpy arrays); grid: node_ids, collider_bits, masses, velocities."""
    n = len(p["flags"])
    out = [header(version), struct.pack("<d", float(time)), _vec(p["flags"], "I")]
    out.append(struct.pack("<Q", n))
    for i in range(n):
        fl = int(p["flags"][i])
        out.append(struct.pack("<ff", p["mass"][i], p["initial_volume"][i]))
        if fl & USE_VISCOSITY:
            out.append(struct.pack("<Bff", 1, p["viscosity_dynamic"][i], p["viscosity_bulk"][i]))
        else:
            out.append(struct.pack("<B", 0))
        if fl & IS_FLUID:
            out.append(struct.pack("<Iif", 1, int(p["exponent"][i]), p["bulk_modulus"][i]))
        else:
            out.append(struct.pack("<Iff", 0, p["mu"][i], p["lambda_"][i]))
            if fl & USE_SAND_ALPHA:
                out.append(struct.pack("<Bf", 1, p["sand_alpha"][i]))
            else:
                out.append(struct.pack("<B", 0))
    for name, fmt in [("elastic_energies", "f"), ("collider_bits", "I"), ("positions", "f"),
                      ("position_gradients", "f"), ("velocities", "f"), ("velocity_gradients", "f"),
                      ("initial_positions", "f")]:
        out.append(_vec(p[name], fmt))
    if grid is None:
        out.append(struct.pack("<B", 0))
    else:
        out.append(struct.pack("<B", 1))
        for name, fmt in [("node_ids", "i"), ("collider_bits", "I"), ("masses", "f"), ("velocities", "f")]:
            out.append(_vec(grid[name], fmt))
    return b"".join(out)


class _Reader:
    def __init__(self, data: bytes):
        self.d, self.o = data, 0

    def take(self, fmt: str):
        v = struct.unpack_from("<" + fmt, self.d, self.o)
        self.o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def vec(self, fmt: str, width: int, dtype):
        n = self.take("Q")
        a = np.frombuffer(self.d, dtype=dtype, count=n * width, offset=self.o).copy()
        self.o += a.nbytes
        return a.reshape(n, width) if width > 1 else a


def decode(data: bytes, version: str):
    """(time, particle dict, grid dict or None) of a frame file's bytes."""
    assert data[:32] == MAGIC, "magic bytes mismatch"
    assert data[32:96] == header(version)[32:], "version mismatch"
    r = _Reader(data)
    r.o = 96
    time = r.take("d")
    p = {"flags": r.vec("I", 1, np.uint32)}
    n = r.take("Q")
    cols = {k: np.zeros(n, np.float32) for k in ["mass", "initial_volume", "viscosity_dynamic", "viscosity_bulk",
                                                  "mu", "lambda_", "sand_alpha", "bulk_modulus"]}
    cols["exponent"] = np.zeros(n, np.int32)
    for i in range(n):
        cols["mass"][i], cols["initial_volume"][i] = r.take("ff")
        if r.take("B"):
            cols["viscosity_dynamic"][i], cols["viscosity_bulk"][i] = r.take("ff")
        if r.take("I") == 1:
            cols["exponent"][i], cols["bulk_modulus"][i] = r.take("if")
        else:
            cols["mu"][i], cols["lambda_"][i] = r.take("ff")
            if r.take("B"):
                cols["sand_alpha"][i] = r.take("f")
    p.update(cols)
    for name, fmt, width, dt in [("elastic_energies", "f", 1, np.float32), ("collider_bits", "I", 1, np.uint32),
                                 ("positions", "f", 3, np.float32), ("position_gradients", "f", 9, np.float32),
                                 ("velocities", "f", 3, np.float32), ("velocity_gradients", "f", 9, np.float32),
                                 ("initial_positions", "f", 3, np.float32)]:
        p[name] = r.vec(fmt, width, dt)
    grid = None
    if r.take("B"):
        grid = {"node_ids": r.vec("i", 3, np.int32), "collider_bits": r.vec("I", 1, np.uint32),
                "masses": r.vec("f", 1, np.float32), "velocities": r.vec("f", 3, np.float32)}
    assert r.o == len(data), "trailing bytes"
    return time, p, grid
