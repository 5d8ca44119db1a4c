"""rk_sort_keys_noalloc (static device scratch, no allocation) against
rk_sort_keys (allocating) through the C ABI, on the GPU.

Both entry points run the same stable radix sort, so their outputs must be
bit-identical.  Two calls in a row check that the shared scratch left by the
first call does not leak into the second."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 19


def _keys(n, seed, lo, hi):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 2 ** 63 - 1, n, dtype=np.int64).view(np.uint64)
    if hi - lo < 64:
        # few distinct values in the sorted field (and random bits outside it,
        # above hi_bit too, which must not take part in the order): checks
        # stability and the masking of the last digit
        a = (a & ~np.uint64(((1 << (hi - lo)) - 1) << lo)) | (
            (rng.integers(0, min(97, 1 << (hi - lo)), n).astype(np.uint64)) << np.uint64(lo))
    return a.view(np.int64)


def _stable_ref(host, lo, hi):
    a = host.view(np.uint64)
    mask = np.uint64((1 << (hi - lo)) - 1) if hi - lo < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    return a[np.argsort((a >> np.uint64(lo)) & mask, kind="stable")]


def test_noalloc_matches_allocating_sort_twice(gpu_lib):
    import torch
    lib = gpu_lib.load()
    cases = [(300001, 0, 64, 11), (MAX_KEYS, 27, 51, 12), (4097, 0, 48, 13), (70001, 3, 13, 14), (5000, 0, 4, 15)]
    for call in range(2):
        for n, lo, hi, seed in cases:
            host = _keys(n, seed + 100 * call, lo, hi)
            a = torch.from_numpy(host.copy()).cuda()
            b = torch.from_numpy(host.copy()).cuda()
            torch.cuda.synchronize()
            assert lib.rk_sort_keys(ctypes.c_void_p(a.data_ptr()), n, lo, hi, None) == 0
            rc = lib.rk_sort_keys_noalloc(ctypes.c_void_p(b.data_ptr()), n, lo, hi, None)
            torch.cuda.synchronize()
            assert rc == 0
            assert torch.equal(a, b), (call, n, lo, hi)
            assert np.array_equal(b.cpu().numpy().view(np.uint64), _stable_ref(host, lo, hi))


def test_noalloc_rejects_oversize_and_bad_args(gpu_lib):
    import torch
    lib = gpu_lib.load()
    t = torch.zeros(MAX_KEYS + 1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    assert lib.rk_sort_keys_noalloc(ctypes.c_void_p(t.data_ptr()), MAX_KEYS + 1, 0, 64, None) == -3
    assert lib.rk_sort_keys_noalloc(ctypes.c_void_p(t.data_ptr()), 10, 8, 8, None) == -1
    assert lib.rk_sort_keys_noalloc(None, 10, 0, 64, None) == -1
    assert lib.rk_sort_keys_noalloc(None, 0, 0, 64, None) == 0


def test_noalloc_call_allocates_nothing(gpu_lib):
    """The property the entry point exists for: once the first call on the
    device has done its set-up, a call changes the device's free memory by
    nothing (cudaMemGetInfo before and after)."""
    import torch
    lib = gpu_lib.load()
    host = _keys(MAX_KEYS, 21, 0, 64)
    t = torch.from_numpy(host).cuda()
    torch.cuda.synchronize()
    assert lib.rk_sort_keys_noalloc(ctypes.c_void_p(t.data_ptr()), MAX_KEYS, 0, 64, None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        assert lib.rk_sort_keys_noalloc(ctypes.c_void_p(t.data_ptr()), MAX_KEYS, 0, 64, None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
