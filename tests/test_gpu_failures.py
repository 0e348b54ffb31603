"""Failure detection without a GPU fault.

  - A bounded tensor-core wait that runs out: sv_debug_closure_wait_timeout
    runs the learned closure's own wait machinery against an MMA commit
    that is never issued (a flag that nothing sets).  The kernel must
    return, raise the closure's timeout counter and leave the context
    usable; the next sv_step reports the timeout as a fatal error.
  - A cancel set from another host thread in the middle of a long sv_step
    (the reference's Harness::check, xpu/src/harness.rs:65-79, polled while
    waiting on the GPU like gpu_state.rs:509-522): the call returns with
    SV_STATUS_CANCELED after a partial run, its substep count matches the
    handle's time, and the state still downloads and keeps stepping.
"""

import threading
import time

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Harness, scenes
from squishy_volumes_gb300._abi import SV_STATUS_CANCELED, SV_TOMBSTONED, SvError

pytestmark = pytest.mark.gpu


def test_closure_wait_timeout_returns_and_is_reported(cuda_lib):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    before = gpu.download()
    t0 = time.perf_counter()
    # about 10 us of waiting at 2 GHz, twice (the wait and ctl_finish's)
    assert cuda_lib.sv_debug_closure_wait_timeout(gpu._h, 20000) == 0
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(SvError, match="tensor-core wait"):
        gpu.step(2, s.dt, s.gravity)
    # the context is usable: the handle downloads, a new handle steps
    out = gpu.download()
    assert np.all(np.isfinite(out.positions)) and out.n == before.n
    gpu.close()
    other = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    assert other.step(3, s.dt, s.gravity) == (0, 3)
    other.close()


def test_closure_wait_timeout_rejects_bad_limits(cuda_lib):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    assert cuda_lib.sv_debug_closure_wait_timeout(gpu._h, 0) == -1
    assert cuda_lib.sv_debug_closure_wait_timeout(gpu._h, 10**10) == -1
    assert cuda_lib.sv_debug_closure_wait_timeout(None, 1000) == -1
    gpu.close()


def test_cancel_from_another_thread_mid_call(cuda_lib):
    s = scenes.three_boxes_1m()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    assert gpu.step(4, s.dt, s.gravity) == (0, 4)  # warm-up: binning, graphs
    t_before = gpu.time
    harness = Harness()
    n = 200_000  # far more than run before the cancel arrives
    result = {}

    def run():
        result["r"] = gpu.step(n, s.dt, s.gravity, harness=harness)

    th = threading.Thread(target=run)
    t0 = time.perf_counter()
    th.start()
    time.sleep(0.3)
    harness.cancel()
    th.join(timeout=60)
    elapsed = time.perf_counter() - t0
    assert not th.is_alive()
    status, done = result["r"]
    assert status & SV_STATUS_CANCELED
    assert 0 < done < n
    # the call returned within a few chunks of the cancel
    assert elapsed < 0.3 + 1.0, elapsed
    # the handle's time advances by the float32 dt of the C ABI per substep
    assert gpu.time == pytest.approx(t_before + done * float(np.float32(s.dt)), rel=1e-9)
    assert gpu.stats()["substeps"] == 4 + done
    out = gpu.download()
    assert np.all(np.isfinite(out.positions[(out.flags & SV_TOMBSTONED) == 0]))
    # and it keeps stepping from there
    assert gpu.step(3, s.dt, s.gravity) == (0, 3)
    gpu.close()


def test_cancel_before_the_call_runs_nothing(cuda_lib):
    s = scenes.small_mixed()
    gpu = CudaState.from_io_state(s.io_state, s.consts, s.extras)
    harness = Harness()
    harness.cancel()
    status, done = gpu.step(10, s.dt, s.gravity, harness=harness)
    assert status & SV_STATUS_CANCELED and done == 0
    gpu.close()
