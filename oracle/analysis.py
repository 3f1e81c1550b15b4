"""numpy restatement of the reference DLL's analysis functions (test infrastructure).

* ``pes`` follows window_analysis (1DTDSE/sources/tools.c:206-316): grid x_k = k dx - 0.5 num_r dx
  (:231, :246), for every energy E_i = E_start + i Estep two Numerov-tridiagonal solves
  (Inv_Tridiagonal_Matrix_complex_Numerov, tridiag.c:251-274, and the Thomas sweep of
  Inv_Tridiagonal_Matrix_complex, tridiag.c:26-70) with
      diagonal      10 (E_i -/+ dE - V_j)/12 - 1/dx^2  -/+ i 10 dE/12
      sub-diagonal  (E_i -/+ dE - V_j)/12 + 0.5/dx^2   -/+ i dE/12   (dinf[j], row j+1)
      super-diag.   (E_i -/+ dE - V_{j+1})/12 + 0.5/dx^2 -/+ i dE/12 (dsup[j], row j)
  the second solve on the first one's result, and PES_i = dx dE^4 sum_j |u2_j|^2 (:296-299).
  Vectorised over energies (the Thomas recurrence runs over rows).
* ``gabor`` follows GaborTransform (1DTDSE/sources/tools_fftw3.c:158-213): window
  exp(-((j dt - (t_min + i dt_G))/a)^2), dt_G = (t_max - t_min)/N_G, real DFT (numpy),
  dt/sqrt(2 pi) |DFT_k| for k < N_freq.
"""
import numpy as np


def potential(x, a):
    """Soft-core potential (tools.c:91-95)."""
    return -1.0 / np.sqrt(a * a + x * x)


def _numerov_solve(dinf, d, dsup, p):
    """Inv_Tridiagonal_Matrix_complex_Numerov on [n, nE] complex arrays (rows first)."""
    n = p.shape[0]
    r = np.empty_like(p)
    r[0] = 10 * p[0] / 12. + p[1] / 12.
    r[1:n - 1] = 10 * p[1:n - 1] / 12. + (p[2:n] + p[0:n - 2]) / 12.
    r[n - 1] = 10 * p[n - 1] / 12. + p[n - 2] / 12.
    u = np.empty_like(p)
    gam = np.zeros_like(p)
    bet = d[0]
    u[0] = r[0] / bet
    for j in range(1, n):
        gam[j] = dsup[j - 1] / bet
        bet = d[j] - dinf[j - 1] * gam[j]
        u[j] = (r[j] - dinf[j - 1] * u[j - 1]) / bet
    for j in range(n - 2, -1, -1):
        u[j] = u[j] - gam[j + 1] * u[j + 1]
    return u


def pes(psi, num_r, dx, a, num_E, dE, Estep, E_start):
    n = num_r + 1
    xmax = 0.5 * num_r * dx
    x = np.arange(n + 1) * dx - xmax
    V = potential(x, a)
    E = E_start + Estep * np.arange(num_E)
    diag, off = 1. / (dx * dx), -0.5 / (dx * dx)
    p = np.repeat(np.asarray(psi, dtype=np.complex128)[:, None], num_E, axis=1)
    for sg in (-1.0, 1.0):
        Es = E[None, :] + sg * dE
        d = (10 * (Es - V[:n, None]) / 12. - diag) + 1j * sg * (10 * dE / 12)
        dinf = ((Es - V[:n, None]) / 12. - off) + 1j * sg * (dE / 12)
        dsup = ((Es - V[1:n + 1, None]) / 12. - off) + 1j * sg * (dE / 12)
        p = _numerov_solve(dinf, d, dsup, p)
    return (np.abs(p) ** 2).sum(axis=0) * dx * dE ** 4


def gabor(signal, dt, N, N_freq, N_G, t_min, t_max, a):
    """Rows [N_G][N_freq] as the reference returns them."""
    ia = 1.0 / a
    dt_G = (t_max - t_min) / N_G
    j = np.arange(N)
    out = np.empty((N_G, N_freq))
    s = np.asarray(signal, dtype=np.float64)[:N]
    for i in range(N_G):
        w = np.exp(-(ia * (j * dt - (t_min + i * dt_G))) ** 2) * s
        out[i] = dt / np.sqrt(2 * np.pi) * np.abs(np.fft.rfft(w)[:N_freq])
    return out
