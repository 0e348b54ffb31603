"""Frame files and the frame cache with host frames (CPU only: no device
calls).  The library's writer is checked against a hand-assembled
known-answer byte string and against the oracle's independent restatement of
the bincode layout; its reader against the restatement's bytes; the cache
against its own files.  Mirrors the reference's checks of the header
(file_util/src/lib.rs:101-157: wrong magic, wrong version)."""

import os

import numpy as np
import pytest

from oracle import frame_file as ref_ff
from squishy_volumes_gb300 import GridNodes, IoState, Particles
from squishy_volumes_gb300._abi import (SV_IS_FLUID, SV_IS_SOLID, SV_TOMBSTONED, SV_USE_SAND_ALPHA, SV_USE_VISCOSITY,
                                        SvError)
from squishy_volumes_gb300.frames import FRAME_VERSION, FrameCache, read_frame, write_frame

HEADER = b"Squishy Volumes Frame File Magic" + b"0.3.4" + bytes(59)

# One solid particle with viscosity and a sand alpha, no grid, time 0.25,
# field by field (little endian; u64 Vec lengths; u8 Option tags; u32 enum
# variant index).
KAT_BODY = bytes.fromhex(
    "000000000000d03f"                                      # time: f64 0.25
    "0100000000000000" "0d000000"                           # flags: [SOLID | VISCOSITY | SAND_ALPHA]
    "0100000000000000"                                      # parameters: Vec of 1
    "00000040" "0000003f"                                   #   mass 2.0, initial_volume 0.5
    "01" "0000803e" "0000003e"                              #   viscosity Some { dynamic 0.25, bulk 0.125 }
    "00000000" "00004040" "00008040" "01" "0000403f"        #   Solid { mu 3.0, lambda 4.0, sand_alpha Some(0.75) }
    "0100000000000000" "0000c03f"                           # elastic_energies [1.5]
    "0100000000000000" "01000100"                           # collider_bits [0x10001]
    "0100000000000000" "0000803f" "00000040" "00004040"     # positions [[1, 2, 3]]
    "0100000000000000" "0000803f" "00000000" "00000000"     # position_gradients [I] (column major)
    "00000000" "0000803f" "00000000"
    "00000000" "00000000" "0000803f"
    "0100000000000000" "0000003f" "00000000" "00000000"     # velocities [[0.5, 0, 0]]
    "0100000000000000" + "00000000" * 9 +                   # velocity_gradients [0]
    "0100000000000000" "0000803f" "00000040" "00004040"     # initial_positions [[1, 2, 3]]
    "00"                                                    # grid_nodes: None
)


def _particles(**kw):
    return Particles(**kw)


def one_particle():
    x = np.array([[1.0, 2.0, 3.0]], np.float32)
    return IoState(0.25, _particles(
        flags=np.array([SV_IS_SOLID | SV_USE_VISCOSITY | SV_USE_SAND_ALPHA], np.uint32),
        positions=x, position_gradients=np.eye(3, dtype=np.float32).reshape(1, 9),
        velocities=np.array([[0.5, 0.0, 0.0]], np.float32), velocity_gradients=np.zeros((1, 9), np.float32),
        mass=[2.0], initial_volume=[0.5], viscosity_dynamic=[0.25], viscosity_bulk=[0.125], mu=[3.0],
        lambda_=[4.0], sand_alpha=[0.75], exponent=[0], bulk_modulus=[0.0], elastic_energies=[1.5],
        collider_bits=np.array([0x10001], np.uint32), initial_positions=x.copy()))


def random_state(rng, n, m, grid=True):
    flags = rng.choice([SV_IS_SOLID, SV_IS_SOLID | SV_USE_SAND_ALPHA, SV_IS_FLUID | SV_USE_VISCOSITY,
                        SV_IS_SOLID | SV_USE_VISCOSITY, SV_IS_FLUID | SV_TOMBSTONED], n).astype(np.uint32)
    f32 = lambda *s: rng.standard_normal(s).astype(np.float32)  # noqa: E731
    solid, fluid = (flags & SV_IS_FLUID) == 0, (flags & SV_IS_FLUID) != 0
    visc, sand = (flags & SV_USE_VISCOSITY) != 0, (flags & SV_USE_SAND_ALPHA) != 0
    p = _particles(
        flags=flags, positions=f32(n, 3), position_gradients=f32(n, 9), velocities=f32(n, 3),
        velocity_gradients=f32(n, 9), mass=np.abs(f32(n)), initial_volume=np.abs(f32(n)),
        viscosity_dynamic=np.where(visc, f32(n), 0).astype(np.float32),
        viscosity_bulk=np.where(visc, f32(n), 0).astype(np.float32),
        mu=np.where(solid, f32(n), 0).astype(np.float32), lambda_=np.where(solid, f32(n), 0).astype(np.float32),
        sand_alpha=np.where(sand, f32(n), 0).astype(np.float32),
        exponent=np.where(fluid, rng.integers(1, 9, n), 0).astype(np.int32),
        bulk_modulus=np.where(fluid, f32(n), 0).astype(np.float32), elastic_energies=f32(n),
        collider_bits=rng.integers(0, 1 << 20, n).astype(np.uint32), initial_positions=f32(n, 3))
    g = None
    if grid:
        g = GridNodes(rng.integers(-50, 50, (m, 3)).astype(np.int32), rng.integers(0, 4, m).astype(np.uint32),
                      np.abs(f32(m)), f32(m, 3))
    return IoState(float(rng.random()), p, g)


def as_dicts(io):
    p = {k: getattr(io.particles, k) for k in ["flags", "mass", "initial_volume", "viscosity_dynamic",
                                                "viscosity_bulk", "mu", "lambda_", "sand_alpha", "exponent",
                                                "bulk_modulus", "elastic_energies", "collider_bits", "positions",
                                                "position_gradients", "velocities", "velocity_gradients",
                                                "initial_positions"]}
    g = None
    if io.grid_nodes is not None:
        g = {"node_ids": io.grid_nodes.node_ids, "collider_bits": io.grid_nodes.collider_bits,
             "masses": io.grid_nodes.masses, "velocities": io.grid_nodes.velocities}
    return p, g


def assert_same(a: IoState, b: IoState):
    assert a.time == b.time
    for k in ["flags", "mass", "initial_volume", "viscosity_dynamic", "viscosity_bulk", "mu", "lambda_",
              "sand_alpha", "exponent", "bulk_modulus", "elastic_energies", "collider_bits", "positions",
              "position_gradients", "velocities", "velocity_gradients", "initial_positions"]:
        np.testing.assert_array_equal(getattr(a.particles, k), getattr(b.particles, k), err_msg=k)
    assert (a.grid_nodes is None) == (b.grid_nodes is None)
    if a.grid_nodes is not None:
        for k in ["node_ids", "collider_bits", "masses", "velocities"]:
            np.testing.assert_array_equal(getattr(a.grid_nodes, k), getattr(b.grid_nodes, k), err_msg=k)


def test_known_answer_bytes(cuda_lib, tmp_path):
    io = one_particle()
    path = tmp_path / "frame_00000.bin"
    assert write_frame(path, io) == len(HEADER) + len(KAT_BODY)
    assert path.read_bytes() == HEADER + KAT_BODY
    p, g = as_dicts(io)
    assert ref_ff.encode(io.time, p, g, FRAME_VERSION) == HEADER + KAT_BODY
    assert not list(tmp_path.glob("*.temp"))  # written beside, then renamed


@pytest.mark.parametrize("n,m,grid", [(0, 0, False), (0, 0, True), (1, 1, True), (257, 1000, True), (1000, 0, False)])
def test_writer_matches_the_restatement_and_round_trips(cuda_lib, tmp_path, n, m, grid):
    io = random_state(np.random.default_rng(n + m), n, m, grid)
    path = tmp_path / "f.bin"
    write_frame(path, io)
    p, g = as_dicts(io)
    data = path.read_bytes()
    assert data == ref_ff.encode(io.time, p, g, FRAME_VERSION)
    assert_same(read_frame(path), io)
    t, p2, g2 = ref_ff.decode(data, FRAME_VERSION)
    assert t == io.time and np.array_equal(p2["positions"], io.particles.positions)


def test_reader_reads_the_restatement(cuda_lib, tmp_path):
    io = random_state(np.random.default_rng(5), 300, 40)
    p, g = as_dicts(io)
    path = tmp_path / "f.bin"
    path.write_bytes(ref_ff.encode(io.time, p, g, "custom-1"))
    assert_same(read_frame(path, version="custom-1"), io)


def test_header_and_truncation_errors(cuda_lib, tmp_path):
    io = random_state(np.random.default_rng(6), 20, 5)
    good = tmp_path / "good.bin"
    write_frame(good, io)
    data = good.read_bytes()
    bad_magic = tmp_path / "magic.bin"
    bad_magic.write_bytes(b"X" + data[1:])
    with pytest.raises(SvError, match="magic"):
        read_frame(bad_magic)
    with pytest.raises(SvError, match="version mismatch, found 0.3.4"):
        read_frame(good, version="0.3.5")
    cut = tmp_path / "cut.bin"
    cut.write_bytes(data[:-7])
    with pytest.raises(SvError, match="truncated"):
        read_frame(cut)
    with pytest.raises(SvError, match="64 bytes"):
        write_frame(tmp_path / "v.bin", io, version="x" * 65)


def test_cache_writes_numbered_frames(cuda_lib, tmp_path):
    rng = np.random.default_rng(7)
    frames = [random_state(rng, 100, 10 * k, grid=k > 0) for k in range(4)]
    with FrameCache(tmp_path, frames[0].particles, first_frame=3) as cache:
        for io in frames:
            cache.store_io_state(io)
        cache.flush()
        count, nbytes = cache.info()
    assert count == 4
    names = sorted(os.listdir(tmp_path))
    assert names == [f"frame_{k:05d}.bin" for k in range(3, 7)]
    assert nbytes == sum((tmp_path / nm).stat().st_size for nm in names)
    for k, io in enumerate(frames):
        assert_same(read_frame(tmp_path / f"frame_{k + 3:05d}.bin"), io)


def test_cache_reports_a_failed_writer(cuda_lib, tmp_path):
    io = random_state(np.random.default_rng(8), 10, 0, grid=False)
    cache = FrameCache(tmp_path / "missing_dir", io.particles)
    cache.store_io_state(io)
    with pytest.raises(SvError, match="cannot create"):
        cache.flush()
    with pytest.raises(SvError):
        cache.check()
    with pytest.raises(SvError):
        cache.store_io_state(io)
    with pytest.raises(SvError):
        cache.close()


def test_prepare_host_keeps_contents(cuda_lib):
    """sv_prepare_host maps the pages of host arrays without changing them
    (no device involved)."""
    import ctypes as ct

    rng = np.random.default_rng(9)
    arrays = [rng.standard_normal(n).astype(np.float32) for n in (1, 1000, 3_000_000)]
    arrays.append(np.empty(2_000_000, np.uint32))  # fresh pages
    arrays[-1][:] = 7
    copies = [a.copy() for a in arrays]
    ptrs = (ct.c_void_p * 5)(*[a.ctypes.data for a in arrays], None)
    sizes = (ct.c_uint64 * 5)(*[a.nbytes for a in arrays], 64)
    assert cuda_lib.sv_prepare_host(ptrs, sizes, 5) == 0  # NULL entries are skipped
    for a, c in zip(arrays, copies):
        np.testing.assert_array_equal(a, c)
    assert cuda_lib.sv_prepare_host(None, None, 0) == 0
    assert cuda_lib.sv_prepare_host(None, sizes, 1) == -1
