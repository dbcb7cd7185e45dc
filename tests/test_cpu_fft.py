"""The oracle's CPU FFT (oracle/qs_fft.c) against numpy in double precision."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle

SIZES = list(range(1, 40)) + [64, 97, 128, 149, 256, 264, 298, 306, 307, 384, 512, 563, 768, 1024]


@pytest.fixture(scope="module")
def lib():
    oracle.build()
    L = ctypes.CDLL(oracle.LIB_PATH)
    L.qs_fft1d_get.restype = ctypes.c_void_p
    L.qs_fft1d_get.argtypes = [ctypes.c_int]
    L.qs_fft1d_exec.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.qs_fftnd_c128.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_ssize_t, ctypes.c_void_p,
                                ctypes.c_int]
    return L


@pytest.mark.parametrize("n", SIZES)
def test_fft1d(lib, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for sign in (-1, 1):
        y = x.copy()
        lib.qs_fft1d_exec(lib.qs_fft1d_get(n), y.ctypes.data, sign, None)
        ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * n
        assert np.abs(y - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("dims", [(4, 6), (306, 264), (3, 5, 7), (307, 298)])
def test_fftnd(lib, dims):
    rng = np.random.default_rng(7)
    x = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
    y = np.ascontiguousarray(x.copy())
    d = (ctypes.c_int * len(dims))(*dims)
    lib.qs_fftnd_c128(len(dims), d, 1, 0, y.ctypes.data, -1)
    ref = np.fft.fftn(x)
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()
