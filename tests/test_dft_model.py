"""CPU check of the device DFT's index arithmetic (tests/dft_model.py restates the plan and the
passes of mma_gb300/csrc/dft.cu) against numpy.fft, before the kernels run on a GPU: Stockham
passes for every radix order the plans produce, Bluestein for lengths that are not 7-smooth, the
even-length real packing (r2c) and its inverse (c2r, with the DC and Nyquist imaginary parts
ignored as FFTW does), and odd lengths."""
import numpy as np
import pytest

from tests import dft_model as D


@pytest.mark.parametrize("M", [2, 3, 4, 5, 7, 8, 12, 30, 35, 56, 105, 128, 384, 2205, 4480])
def test_stockham_passes(M):
    rng = np.random.default_rng(M)
    x = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    ref = np.fft.fft(x)
    got = D.stockham_vec(x, D.twiddles(M), D.radices(M))
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    if M <= 128:  # the per-butterfly loop form, literally as the kernels index
        got = D.stockham(x, D.twiddles(M), D.radices(M))
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("L", [7, 11, 97, 1103, 2206])
def test_complex_dft_by_plan(L):
    rng = np.random.default_rng(L)
    z = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    p = D.plan(L)
    assert p["bluestein"] == (not D.is_smooth(L))
    assert p["M"] >= (2 * L - 1 if p["bluestein"] else L) and D.is_smooth(p["M"])
    ref = np.fft.fft(z)
    assert np.abs(D.cdft(z, p) - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("n", [2, 3, 4, 5, 17, 441, 1000, 4410, 4412, 4413])
def test_real_transforms(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    R = np.fft.rfft(x)
    X = D.rfft(x)
    assert np.abs(X - R).max() <= 1e-13 * np.abs(R).max()
    Xp = R.copy()
    Xp[0] += 0.3j  # ignored, as FFTW's c2r ignores it
    if n % 2 == 0:
        Xp[-1] += 0.7j
    y = D.irfft(Xp, n)
    ref = np.fft.irfft(R, n) * n
    assert np.abs(y - ref).max() <= 1e-13 * np.abs(ref).max()
