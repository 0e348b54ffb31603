"""Upload and download by kernels that access the caller's pageable host
arrays (sv_transfer.cu) against the staged copies: the same bits, for both
position forms, batched scenes, tombstoned particles and collider bits."""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, IoState, scenes
from squishy_volumes_gb300._abi import SV_TOMBSTONED
from squishy_volumes_gb300.state import BatchedCudaState

pytestmark = pytest.mark.gpu

FIELDS = ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "elastic_energies",
          "collider_bits", "plastic_j"]


def same(a, b):
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)


def with_tombstones(p):
    p = p.copy()
    p.flags[::7] |= SV_TOMBSTONED
    p.collider_bits = (np.arange(p.n) % 5 == 0).astype(np.uint32) * 0x10001
    return p


@pytest.mark.parametrize("form", [0, 1])
def test_upload_paths_give_the_same_state(cuda_lib, form):
    s = scenes.small_mixed()
    p = with_tombstones(s.io_state.particles)
    direct = CudaState.from_io_state(IoState(0.0, p), s.consts, Extras(position_form=form, host_transfer=0))
    staged = CudaState.from_io_state(IoState(0.0, p), s.consts, Extras(position_form=form, host_transfer=1))
    assert not staged.set_host_transfer(1)
    uses_direct = direct.set_host_transfer(0)
    if not uses_direct:
        pytest.skip("the device cannot access pageable host memory")
    same(direct.download(), staged.download())
    # positions round-trip exactly through the cell form, as through the staged path
    if form == 0:
        np.testing.assert_array_equal(direct.download().positions, p.positions)
    direct.close(), staged.close()


@pytest.mark.parametrize("form", [0, 1])
def test_download_paths_agree_after_stepping(cuda_lib, form):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(IoState(0.0, with_tombstones(s.io_state.particles)), s.consts,
                                  Extras(position_form=form))
    assert gpu.step(25, s.dt, s.gravity)[0] == 0
    if not gpu.set_host_transfer(0):
        pytest.skip("the device cannot access pageable host memory")
    a = gpu.download()
    gpu.set_host_transfer(1)
    b = gpu.download()
    same(a, b)
    assert (a.collider_bits[(a.flags & SV_TOMBSTONED) != 0] != 0).any()  # tombstoned keep their initial bits
    gpu.close()


def test_download_paths_agree_with_a_frame_input(cuda_lib, oracle_mod):
    from test_gpu_colliders import _consts, _falling_box, _frame, _quad

    gpu = CudaState.from_io_state(IoState(0.0, _falling_box()), _consts(), Extras())
    V, T, col = _quad(0.45)
    gpu.set_frame_input(_frame(V=V, T=T, col=col))
    assert gpu.step(300, 1e-4, (0, 0, 0)) == (0, 300)
    if not gpu.set_host_transfer(0):
        pytest.skip("the device cannot access pageable host memory")
    a = gpu.download()
    gpu.set_host_transfer(1)
    same(a, gpu.download())
    assert (a.collider_bits != 0).any()
    gpu.close()


def test_batched_scenes_both_paths(cuda_lib):
    batch = scenes.batched_64(n_scenes=4, median=2000.0, lo=1000, hi=5000)
    ios = [sc.io_state for sc in batch]
    cons = [sc.consts for sc in batch]
    direct = BatchedCudaState.from_scenes(ios, cons, Extras(host_transfer=0))
    staged = BatchedCudaState.from_scenes(ios, cons, Extras(host_transfer=1))
    for k in range(len(batch)):
        same(direct.download_scene(k), staged.download_scene(k))
    direct.close(), staged.close()
