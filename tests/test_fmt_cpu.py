"""The exact printf("%.*e") of rk_fmt.cuh (what the device conf text is made
of), built for the host, against Python's correctly rounded formatting (ties
to even, as the C library's default mode) and, for the contact normals'
rounding toward zero, against the exact decimal value truncated (CPU)."""
import ctypes
import decimal
import os
import struct
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fmt(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("fmt") / "libfmt.so")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so, os.path.join(HERE, "fmt_check.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so)
    lib.rk_fmt_e_host.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
    buf = ctypes.create_string_buffer(64)

    def f(x, p, tz=False):
        lib.rk_fmt_e_host(x, p, 1 if tz else 0, buf)
        return buf.value.decode()
    return f


def toward_zero(x, p):
    """printf("%.*e") of x rounded toward zero, from its exact decimal value."""
    if x != x or x in (float("inf"), float("-inf")):
        return "%.*e" % (p, x)
    d = decimal.Decimal(x)
    sign = "-" if (d.is_signed()) else ""
    d = abs(d)
    if d == 0:
        return sign + "%.*e" % (p, 0.0)
    e = d.adjusted()
    q = d.scaleb(-e).quantize(decimal.Decimal(1).scaleb(-p), rounding=decimal.ROUND_DOWN)
    digits = format(q, "f")
    return "%s%se%s%02d" % (sign, digits, "-" if e < 0 else "+", abs(e))


def samples(n, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2 ** 63, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    xs = [struct.unpack("<d", struct.pack("<Q", int(b)))[0] for b in bits]
    xs += list(rng.uniform(-1, 1, n) * 10.0 ** rng.integers(-20, 20, n))
    xs += [0.0, -0.0, 1.0, 0.5, 2.5, 1.5, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, 0.1,
           float("inf"), float("-inf"), 1e16, 9.999999999999999e22, 123456789.5]
    return [x for x in xs if x == x]


@pytest.mark.parametrize("prec", [0, 3, 13, 16, 17])
def test_nearest_matches_printf(fmt, prec):
    for x in samples(20000, prec):
        assert fmt(x, prec) == "%.*e" % (prec, x), (x, prec)


@pytest.mark.parametrize("prec", [13, 16])
def test_toward_zero_matches_the_exact_value_truncated(fmt, prec):
    for x in samples(5000, 100 + prec):
        assert fmt(x, prec, True) == toward_zero(x, prec), (x, prec)


def test_ties_go_to_even(fmt):
    for x, p, want in [(2.5, 0, "2e+00"), (3.5, 0, "4e+00"), (0.125, 1, "1.2e-01"), (0.375, 1, "3.8e-01")]:
        assert fmt(x, p) == want
