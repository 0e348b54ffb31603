"""The allocation-free sort entry point, through the C ABI.

sv_sort_pairs_noalloc serves callers that may not allocate device memory (a
plugin inside an application that owns the whole device-memory budget
through its own pool, or a loop that cannot take the device-wide
synchronisation of an allocation).  Its scratch is a fixed array inside the
library, so it only takes caller-owned device buffers.  It must give the
same permutation as the allocating sv_sort_pairs and as a stable CPU
argsort, call after call (the shared scratch keeps the previous call's
contents), and refuse sizes above its limit.  This file is collected last so
that a failure here leaves every other test already run.
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20


def _noalloc(lib):
    fn = lib.sv_sort_pairs_noalloc
    fn.restype = ct.c_int
    fn.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint64, ct.c_void_p, ct.c_char_p, ct.c_uint64]
    return fn


def _run(fn, torch, keys: np.ndarray) -> np.ndarray:
    d_keys = torch.from_numpy(keys.view(np.int32)).cuda()
    d_perm = torch.full((keys.shape[0],), -1, dtype=torch.int32, device="cuda")
    err = ct.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(d_keys.data_ptr(), d_perm.data_ptr(), keys.shape[0], stream, err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return d_perm.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_twice(cuda_lib):
    torch = pytest.importorskip("torch")
    from squishy_volumes_gb300 import sort_pairs

    fn = _noalloc(cuda_lib)
    rng = np.random.default_rng(2024)
    # two calls in a row through the same shared scratch: a full-size call
    # with wide keys, then a smaller one with many equal keys
    first = rng.integers(0, 2**32, MAX_KEYS, dtype=np.uint64).astype(np.uint32)
    second = rng.integers(0, 1000, 250_001).astype(np.uint32)
    for keys in (first, second):
        got = _run(fn, torch, keys)
        np.testing.assert_array_equal(got, sort_pairs(keys))
        # independent of the GPU sort's kernels: the stable CPU argsort
        np.testing.assert_array_equal(got, np.argsort(keys, kind="stable").astype(np.uint32))


def test_noalloc_sort_rejects_oversize(cuda_lib):
    torch = pytest.importorskip("torch")
    fn = _noalloc(cuda_lib)
    n = MAX_KEYS + 1
    d_keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    err = ct.create_string_buffer(256)
    rc = fn(d_keys.data_ptr(), d_perm.data_ptr(), n, None, err, len(err))
    assert rc == -1
    assert b"SV_NOALLOC_MAX_KEYS" in err.value
