"""The oracle's DFTs (oracle/dft.c, also behind the FFTW shim) against numpy.fft."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def dft(oracle_built):
    import oracle

    lib = ctypes.CDLL(oracle.oracle_lib_path())
    dp = ctypes.POINTER(ctypes.c_double)
    for f in (lib.odft_r2c, lib.odft_c2r):
        f.argtypes = [ctypes.c_int, dp, dp]
        f.restype = None
    lib.odft_complex.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int]
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("n", [2, 3, 8, 17, 1024, 4412, 4413, 1103])
def test_r2c_c2r(dft, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    out = np.zeros(2 * (n // 2 + 1))
    dft.odft_r2c(n, _p(x), _p(out))
    ref = np.fft.rfft(x)
    got = out[0::2] + 1j * out[1::2]
    assert np.max(np.abs(got - ref)) < 1e-12 * np.max(np.abs(ref))
    back = np.zeros(n)
    dft.odft_c2r(n, _p(out), _p(back))
    assert np.max(np.abs(back / n - x)) < 1e-13


def test_complex_both_signs(dft):
    rng = np.random.default_rng(1)
    n = 333
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    zi = np.empty(2 * n)
    zi[0::2], zi[1::2] = z.real, z.imag
    out = np.zeros(2 * n)
    dft.odft_complex(n, _p(zi), _p(out), -1)
    assert np.allclose(out[0::2] + 1j * out[1::2], np.fft.fft(z), atol=1e-11)
    dft.odft_complex(n, _p(zi), _p(out), +1)
    assert np.allclose(out[0::2] + 1j * out[1::2], np.fft.ifft(z) * n, atol=1e-11)
