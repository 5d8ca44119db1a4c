"""The NL rebuild's stable radix sort through rk_sort_keys (GPU)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(lib, t, lo, hi):
    import torch
    rc = lib.rk_sort_keys(ctypes.c_void_p(t.data_ptr()), t.numel(), lo, hi, None)
    torch.cuda.synchronize()
    assert rc == 0


@pytest.mark.parametrize("n", [1, 2, 1000, 4096, 4097, 300001])
def test_sort_full_keys(n, gpu_lib):
    import torch
    lib = gpu_lib.load()
    rng = np.random.default_rng(n)
    a = rng.integers(0, 2 ** 63 - 1, n, dtype=np.int64)
    t = torch.from_numpy(a.copy()).cuda()
    _sort(lib, t, 0, 64)
    assert np.array_equal(t.cpu().numpy().view(np.uint64), np.sort(a.view(np.uint64)))


def test_sort_is_stable_on_a_bit_range(gpu_lib):
    """Keys (j << 27 | index) sorted on the j bits only keep index order:
    the j-side list of the neighbour list relies on it."""
    import torch
    lib = gpu_lib.load()
    n = 200000
    rng = np.random.default_rng(5)
    j = rng.integers(0, 5000, n).astype(np.uint64)
    a = (j << np.uint64(27)) | np.arange(n, dtype=np.uint64)
    t = torch.from_numpy(a.view(np.int64).copy()).cuda()
    _sort(lib, t, 27, 51)
    out = t.cpu().numpy().view(np.uint64)
    ref = a[np.argsort(j, kind="stable")]
    assert np.array_equal(out, ref)
