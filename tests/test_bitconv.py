"""The integer-pipe FP32 <-> FP64 conversions of csrc/bitconv.cuh (host and
device code alike) against numpy's casts: random bit patterns over every
exponent, signed zeros, subnormals, the ends of the float range, rounding
ties, overflow to infinity, infinities and NaNs.  The header is compiled for
the host with g++ here (no GPU)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "p4pdes_gb300", "csrc")

SRC = r"""
#include "bitconv.cuh"
extern "C" void conv_f2d(const float *a, double *o, long n) { for (long i = 0; i < n; i++) o[i] = fg::f2d_bits(a[i]); }
extern "C" void conv_d2f(const double *a, float *o, long n) { for (long i = 0; i < n; i++) o[i] = fg::d2f_bits(a[i]); }
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("bitconv")
    src, so = d / "conv.cpp", d / "libconv.so"
    src.write_text(SRC)
    subprocess.run([cxx, "-O2", "-shared", "-fPIC", "-I", HDR, str(src), "-o", str(so)], check=True)
    L = ctypes.CDLL(str(so))
    L.conv_f2d.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
    L.conv_d2f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
    return L


def f2d(L, a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    o = np.empty(a.shape, np.float64)
    L.conv_f2d(a.ctypes.data, o.ctypes.data, a.size)
    return o


def d2f(L, a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    o = np.empty(a.shape, np.float32)
    L.conv_d2f(a.ctypes.data, o.ctypes.data, a.size)
    return o


def same_bits(x, y):
    return np.array_equal(x.view(np.uint64 if x.dtype == np.float64 else np.uint32),
                          y.view(np.uint64 if y.dtype == np.float64 else np.uint32))


def test_float_to_double_is_the_cast(lib):
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 1 << 32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    a = bits.view(np.float32)
    a = a[~np.isnan(a)]
    special = np.array([0.0, -0.0, np.inf, -np.inf, 1e-45, -1e-45, 1.1754942e-38, 1.17549435e-38,
                        3.4028235e38, -3.4028235e38, 1.0, -1.0], dtype=np.float32)
    for x in (a, special):
        assert same_bits(f2d(lib, x), x.astype(np.float64))
    assert np.isnan(f2d(lib, np.array([np.nan], np.float32)))[0]


def test_double_to_float_is_the_cast(lib):
    rng = np.random.default_rng(1)
    # random mantissas over the exponents around and inside the float range
    exp = rng.integers(1023 - 160, 1023 + 140, 2_000_000, dtype=np.uint64)
    man = rng.integers(0, 1 << 52, exp.size, dtype=np.uint64)
    sgn = rng.integers(0, 2, exp.size, dtype=np.uint64) << np.uint64(63)
    a = (sgn | (exp << np.uint64(52)) | man).view(np.float64)
    # rounding ties (the dropped 29 bits exactly half) on odd and even kept
    # mantissas, one ulp either side, and the carry into the exponent
    keep = rng.integers(0, 1 << 23, 10_000, dtype=np.uint64)
    e = rng.integers(1023 - 126, 1023 + 127, keep.size, dtype=np.uint64)
    half = np.uint64(1 << 28)
    base = (e << np.uint64(52)) | (keep << np.uint64(29))
    ties = np.concatenate([base | half, (base | half) + np.uint64(1), (base | half) - np.uint64(1),
                           (e << np.uint64(52)) | np.uint64((1 << 52) - 1)]).view(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, 1e-45, 7e-46, 1.1754942e-38, 1.17549435e-38,
                        3.4028235e38, 3.4028235677973366e38, 3.4028235677973362e38, 3.5e38, -3.5e38,
                        1e300, -1e300, 5e-324, 1.0, -1.0, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24], np.float64)
    with np.errstate(over="ignore"):
        for x in (a, ties, special):
            assert same_bits(d2f(lib, x), x.astype(np.float32))
    assert np.isnan(d2f(lib, np.array([np.nan], np.float64)))[0]
