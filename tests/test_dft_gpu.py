"""The library's own batched real DFTs (mma_dft_r2c / mma_dft_c2r, which the Fourier
interpolation, the spectra and the Gabor transforms use) against numpy.fft, through the C-ABI.

Lengths cover every path: 7-smooth halves (direct Stockham passes), Bluestein's convolution,
odd lengths, the benchmark's series length 4412 (Bluestein over 4480) and field length 4410,
and lengths whose FFT is too long for shared memory (one launch per pass through global
memory).  Rows are strided.  Tolerance: max |error| <= 1e-12 of the largest value, FP64.
"""
import ctypes
from ctypes import POINTER, c_double, c_float, c_int, c_int64, c_void_p

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-12
LENGTHS = [2, 3, 16, 17, 441, 1000, 2206, 4410, 4412, 4413, 8820, 16384, 20002, 30001]


@pytest.fixture(scope="module")
def lib(gpu_lib):
    L = gpu_lib
    L.mma_dft_r2c.argtypes = [c_int, c_void_p, c_int64, c_void_p, c_int64, c_int, c_void_p]
    L.mma_dft_r2c.restype = c_int
    L.mma_dft_c2r.argtypes = [c_int, c_void_p, c_int64, c_int, c_void_p, c_int64, c_int, c_double, c_void_p]
    L.mma_dft_c2r.restype = c_int
    L.mma_dft_plan_info.argtypes = [c_int, POINTER(c_int), POINTER(c_int), POINTER(c_int), POINTER(c_float)]
    L.mma_dft_plan_info.restype = c_int
    return L


def _info(lib, n):
    m, b, t = c_int(), c_int(), c_int()
    ms = (c_float * 2)()
    assert lib.mma_dft_plan_info(n, ctypes.byref(m), ctypes.byref(b), ctypes.byref(t), ms) == 0
    return m.value, b.value, t.value, list(ms)


@pytest.mark.parametrize("n", LENGTHS)
def test_r2c_matches_numpy(lib, n):
    rng = np.random.default_rng(n)
    rows, xs, Xs = 5, n + 3, n // 2 + 4  # strided rows
    x = rng.standard_normal((rows, xs))
    dx = torch.tensor(x, device="cuda")
    dX = torch.full((rows, Xs), complex("nan"), dtype=torch.complex128, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert lib.mma_dft_r2c(n, dx.data_ptr(), xs, dX.data_ptr(), Xs, rows, st) == 0
    torch.cuda.synchronize()
    ref = np.fft.rfft(x[:, :n], axis=1)
    got = dX[:, :n // 2 + 1].cpu().numpy()
    assert np.abs(got - ref).max() <= TOL * np.abs(ref).max()
    m, b, t, ms = _info(lib, n)
    half = n // 2 if n % 2 == 0 else n
    assert b == (m != half)
    assert t in ((256, 512) if m <= 7168 else (0,))
    print("n %d: FFT length %d, bluestein %d, CTA threads %d, probe ms %s" % (n, m, b, t, ms))


@pytest.mark.parametrize("n,nb", [(2, 2), (17, 9), (1000, 501), (4412, 2207), (13230, 2206), (13230, 4411),
                                  (20002, 6000), (30001, 15001)])
def test_c2r_matches_numpy(lib, n, nb):
    """From the first nb bins (the rest zero), times a scale: the Fourier interpolation's use."""
    rng = np.random.default_rng(n + nb)
    rows, Xs, xs = 3, nb + 1, n + 5
    X = rng.standard_normal((rows, Xs)) + 1j * rng.standard_normal((rows, Xs))
    dX = torch.tensor(X, device="cuda")
    dx = torch.full((rows, xs), float("nan"), dtype=torch.float64, device="cuda")
    scale = 1.0 / 4410.0
    st = torch.cuda.current_stream().cuda_stream
    assert lib.mma_dft_c2r(n, dX.data_ptr(), Xs, nb, dx.data_ptr(), xs, rows, scale, st) == 0
    torch.cuda.synchronize()
    full = np.zeros((rows, n // 2 + 1), dtype=np.complex128)
    full[:, :min(nb, n // 2 + 1)] = X[:, :min(nb, n // 2 + 1)]
    ref = np.fft.irfft(full, n, axis=1) * n * scale
    got = dx[:, :n].cpu().numpy()
    assert np.abs(got - ref).max() <= TOL * np.abs(ref).max()


def test_round_trip_interpolates_a_band_limited_field(lib):
    """r2c of 441 samples then c2r to 3 x 441 samples from the same bins (FourInterp with k1 = 3)
    reproduces a band-limited signal at the refined times."""
    n, k1 = 442, 3
    t = np.arange(n) / n
    f = np.cos(2 * np.pi * 5 * t) + 0.3 * np.sin(2 * np.pi * 17 * t)
    tf = np.arange(k1 * n) / (k1 * n)
    ref = np.cos(2 * np.pi * 5 * tf) + 0.3 * np.sin(2 * np.pi * 17 * tf)
    dx = torch.tensor(f[None, :], device="cuda")
    dX = torch.zeros((1, n // 2 + 1), dtype=torch.complex128, device="cuda")
    out = torch.zeros((1, k1 * n), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert lib.mma_dft_r2c(n, dx.data_ptr(), n, dX.data_ptr(), n // 2 + 1, 1, st) == 0
    assert lib.mma_dft_c2r(k1 * n, dX.data_ptr(), n // 2 + 1, n // 2 + 1, out.data_ptr(), k1 * n, 1, 1.0 / n, st) == 0
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy()[0] - ref).max() < 1e-12


def test_plans_refused_during_capture_and_captured_calls_replay(lib):
    """A length planned beforehand runs inside a CUDA graph; a length never planned is refused
    during capture (status 4) instead of allocating."""
    n = 4412
    x = torch.randn(4, n, dtype=torch.float64, device="cuda")
    X = torch.zeros(4, n // 2 + 1, dtype=torch.complex128, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        assert lib.mma_dft_r2c(n, x.data_ptr(), n, X.data_ptr(), n // 2 + 1, 4, s.cuda_stream) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    rcs = []
    with torch.cuda.graph(g):
        st = torch.cuda.current_stream().cuda_stream
        rcs.append(lib.mma_dft_r2c(n, x.data_ptr(), n, X.data_ptr(), n // 2 + 1, 4, st))
        rcs.append(lib.mma_dft_r2c(n + 6, x.data_ptr(), n, X.data_ptr(), n // 2 + 1, 1, st))
    assert rcs == [0, 4]
    X.zero_()
    g.replay()
    torch.cuda.synchronize()
    ref = np.fft.rfft(x.cpu().numpy(), axis=1)
    assert np.abs(X.cpu().numpy() - ref).max() <= TOL * np.abs(ref).max()
