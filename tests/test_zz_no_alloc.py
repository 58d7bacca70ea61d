"""The allocation-free sort, gy_sort_keys_static, against the allocating gy_sort_keys.

Some callers of the sort cannot allocate device memory where they sort (a framework whose
pool owns all device memory, a loop that cannot take the synchronisation cudaFree implies);
gy_sort_keys_static serves them with scratch compiled into the library.  This file is
collected last so that a run stopping at its first failure has already run everything else.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_sort(lib, torch, keys_host, key_bits):
    from graphyt_gb300 import _lib
    d_keys = torch.from_numpy(keys_host).to("cuda")
    d_perm = torch.full((len(keys_host),), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.gy_sort_keys_static(ctypes.c_void_p(d_keys.data_ptr()), len(keys_host), key_bits,
                                 ctypes.c_void_p(d_perm.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == _lib.GY_OK
    stream.synchronize()
    return d_perm.cpu().numpy()


def test_static_sort_matches_allocating_sort_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graphyt_gb300 import _lib
    rng = np.random.default_rng(11)
    # two calls in a row on different inputs, the larger first: the fullest use of the fixed
    # scratch (GY_SORT_STATIC_MAX keys of 31 bits, four radix passes), then a small input
    # with few key bits (two passes), which must not see the first call's leftovers
    cases = [(rng.integers(0, 1 << 31, _lib.GY_SORT_STATIC_MAX, dtype=np.int64).astype(np.int32), 31),
             (np.repeat(rng.integers(0, 5000, 3_001), 8).astype(np.int32), 13)]
    for keys, bits in cases:
        got = _static_sort(gpu_lib, torch, keys, bits)
        want = _lib.sort_keys(keys)  # the allocating entry point
        assert np.array_equal(got, want)
        assert np.array_equal(got, np.argsort(keys, kind="stable"))


def test_static_sort_rejects_oversize_without_gpu_work(gpu_lib):
    from graphyt_gb300 import _lib
    rc = gpu_lib.gy_sort_keys_static(ctypes.c_void_p(1), _lib.GY_SORT_STATIC_MAX + 1, 20, ctypes.c_void_p(1), None)
    assert rc == _lib.GY_ERR_ARG
