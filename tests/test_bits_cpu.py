"""The integer-pipe FP64 <-> FP32 conversions of the mixed form
(rockable_gb300/csrc/rk_bits.cuh), compiled for the host with g++ and checked
against numpy's IEEE conversions on random and edge-case values."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include "rk_bits.cuh"
extern "C" void conv_d2f(const double* a, float* b, long n) { for (long k = 0; k < n; k++) b[k] = rk::d2f(a[k]); }
extern "C" void conv_f2d(const float* a, double* b, long n) { for (long k = 0; k < n; k++) b[k] = rk::f2d(a[k]); }
'''


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("bits")
    src, so = d / "bits.cpp", d / "bits.so"
    src.write_text(SRC)
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "rockable_gb300", "csrc"),
                           str(src), "-o", str(so)])
    L = ctypes.CDLL(str(so))
    for f in (L.conv_d2f, L.conv_f2d):
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
    return L


def d2f(L, a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.empty(a.shape, np.float32)
    L.conv_d2f(a.ctypes.data, b.ctypes.data, a.size)
    return b


def f2d(L, a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.empty(a.shape, np.float64)
    L.conv_f2d(a.ctypes.data, b.ctypes.data, a.size)
    return b


def test_d2f_rounds_to_nearest(lib):
    rng = np.random.default_rng(3)
    a = rng.standard_normal(1_000_000) * np.exp(rng.uniform(-80, 80, 1_000_000))
    got = d2f(lib, a)
    want = a.astype(np.float32)
    normal = (np.abs(a) >= np.finfo(np.float32).tiny) & (np.abs(a) < np.finfo(np.float32).max)
    # identical except at exact ties (round-half-away here, half-even in numpy)
    m = a.view(np.uint64) & np.uint64((1 << 29) - 1)
    tie = m == np.uint64(1 << 28)
    bad = normal & ~tie & (got.view(np.uint32) != want.view(np.uint32))
    assert not bad.any(), a[bad][:5]
    rel = np.abs(got[normal].astype(np.float64) - a[normal]) / np.abs(a[normal])
    assert rel.max() <= 2.0 ** -24


def test_d2f_edges(lib):
    vals = np.array([0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 1e300, -1e300, np.inf, -np.inf, np.nan,
                     np.nextafter(1.0, 0.0), 3.4028234663852886e38, 3.4028235677973366e38, 1.1754943508222875e-38])
    got = d2f(lib, vals)
    assert got[0] == 0 and not np.signbit(got[0]) and got[1] == 0 and np.signbit(got[1])
    assert got[2] == 1 and got[3] == -1
    assert got[4] == 0 and got[5] == 0 and np.signbit(got[5])
    assert got[6] == np.inf and got[7] == -np.inf and got[8] == np.inf and got[9] == -np.inf
    assert np.isnan(got[10])
    assert got[11] == 1.0  # rounds up into the next binade
    assert got[12] == np.float32(3.4028234663852886e38)
    assert got[13] == np.inf
    assert got[14] == np.finfo(np.float32).tiny


def test_f2d_exact(lib):
    rng = np.random.default_rng(4)
    u = rng.integers(0, 2 ** 32, 1_000_000, dtype=np.uint64).astype(np.uint32)
    f = u.view(np.float32)
    got = f2d(lib, f)
    e = (u >> 23) & 0xFF
    normal = (e > 0) & (e < 255)
    assert np.array_equal(got[normal], f[normal].astype(np.float64))
    assert np.all(got[e == 0] == 0) and np.array_equal(np.signbit(got[e == 0]), np.signbit(f[e == 0]))
    inf = (e == 255) & ((u & 0x7FFFFF) == 0)
    nan = (e == 255) & ((u & 0x7FFFFF) != 0)
    assert np.all(np.isinf(got[inf])) and np.all(np.isnan(got[nan]))
