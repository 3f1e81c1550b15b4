"""Batched TDSE analysis on the GPU: photoelectron spectra and Gabor transforms.

``pes`` computes window_analysis (1DTDSE/sources/tools.c:206-316) for many energies at once, one
GPU thread per energy; ``gabor`` computes GaborTransform (1DTDSE/sources/tools_fftw3.c:158-213)
for a batch of signals (for example every instance's dipole acceleration of a TDSE batch).
Inputs and outputs are torch tensors on the GPU; the kernels are in csrc/tdse_analysis.cu.
The reference's single-call host forms are ``TDSE_DLL.compute_PES`` / ``gabor_transform``.
"""
import ctypes
from ctypes import c_double, c_int, c_int64, c_size_t, c_void_p

import numpy as np
import torch

from ._lib import load
from .tdse_batch import _check, _stream_ptr


def _sig():
    lib = load()
    if getattr(lib, "_mma_analysis_sig", False):
        return lib
    lib.mma_tdse_pes_scratch_bytes.argtypes = [c_int, c_int]
    lib.mma_tdse_pes_scratch_bytes.restype = c_size_t
    lib.mma_tdse_pes.argtypes = [c_void_p, c_int, c_double, c_double, c_int, c_double, c_double, c_double, c_void_p,
                                 c_void_p, c_size_t, c_void_p]
    lib.mma_tdse_pes.restype = c_int
    lib.mma_gabor_scratch_bytes.argtypes = [c_int, c_int, c_int]
    lib.mma_gabor_scratch_bytes.restype = c_size_t
    lib.mma_gabor.argtypes = [c_void_p, c_int64, c_int, c_double, c_int, c_int, c_int, c_double, c_double, c_double,
                              c_void_p, c_void_p, c_size_t, c_void_p]
    lib.mma_gabor.restype = c_int
    lib._mma_analysis_sig = True
    return lib


def _on_device(t):
    """The tensor on the current CUDA device (a host tensor is copied): the kernels take device
    pointers only, so a host pointer never reaches them."""
    return t if t.is_cuda else t.to(torch.device("cuda", torch.cuda.current_device()))


def pes(psi, num_r, dx, trg_a, E_start=-0.6, num_E=10000, epsilon=5e-4, Estep=5e-4, chunk=16384, stream=None):
    """Photoelectron spectrum of one wavefunction (complex tensor of num_r + 1 values; a host tensor is copied to the GPU):
    returns (E grid numpy, PES float64 cuda tensor [num_E]).  Energies run `chunk` at a time."""
    lib = _sig()
    p = _on_device(psi).to(torch.complex128).contiguous()
    if p.numel() != num_r + 1:
        raise ValueError("psi must have num_r + 1 values")
    out = torch.empty(int(num_E), dtype=torch.float64, device=p.device)
    sb = int(lib.mma_tdse_pes_scratch_bytes(int(num_r), int(min(chunk, num_E))))
    sc = torch.empty(sb, dtype=torch.uint8, device=p.device)
    _check(lib.mma_tdse_pes(p.data_ptr(), int(num_r), float(dx), float(trg_a), int(num_E), float(epsilon),
                            float(Estep), float(E_start), out.data_ptr(), sc.data_ptr(), sb, _stream_ptr(stream)),
           "mma_tdse_pes")
    return np.linspace(E_start, E_start + (num_E - 1) * Estep, int(num_E)), out


def gabor(signals, dt, omega_max, t_min, t_max, N_G, a=8.0, stream=None):
    """|Gabor transform| of each row of ``signals`` (float64 cuda tensor [n_sig, N]):
    returns (t grid [N_G], omegas [N_freq], |G| cuda tensor [n_sig, N_G, N_freq]), with the
    frequency selection of PythonTDSE.gabor_transform (2 pi fftfreq(N, dt) <= omega_max)."""
    lib = _sig()
    s = _on_device(signals).to(torch.float64)
    if s.dim() == 1:
        s = s[None]
    s = s.contiguous()
    n_sig, N = s.shape
    omegas = 2 * np.pi * np.fft.fftfreq(N, dt)[0:N // 2]
    sel = omegas <= omega_max
    n_freq = int(np.count_nonzero(sel))
    out = torch.empty(n_sig, int(N_G), n_freq, dtype=torch.float64, device=s.device)
    sb = int(lib.mma_gabor_scratch_bytes(n_sig, N, int(N_G)))
    sc = torch.empty(sb, dtype=torch.uint8, device=s.device)
    _check(lib.mma_gabor(s.data_ptr(), N, n_sig, float(dt), N, n_freq, int(N_G), float(t_min), float(t_max), float(a),
                         out.data_ptr(), sc.data_ptr(), sb, _stream_ptr(stream)), "mma_gabor")
    return np.linspace(t_min, t_max, int(N_G)), omegas[sel], out
