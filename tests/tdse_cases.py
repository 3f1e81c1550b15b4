"""Shared TDSE test inputs (seeded, synthetic): sin^2-envelope 800 nm pulses on soft-Coulomb grids."""
import numpy as np

A_CONFIG = np.sqrt(1.68)  # soft-Coulomb a of the benchmark configurations (a^2 = 1.68)
OMEGA0 = 0.057            # 800 nm in atomic units


def sin2_pulse(n_cycles, E0=0.0534, omega=OMEGA0, dt=0.25, cep=0.0, even=True, skip_first=False, exact_dt=False):
    """Field sampled at ~dt on t in [0, T], T = n_cycles 2 pi/omega; an even sample count
    keeps the reference's last-step field read inside its interpolation buffer.

    exact_dt samples at t = j dt exactly (the linspace grid's spacing T/(n-1) is slightly below
    dt, which matters where the reference derives its refinement factor from the spacing).

    skip_first drops the t = 0 sample (where the field is exactly 0).  The reference's
    zero gate tests f[0] f[1] <= 0 on its Fourier-interpolated field, so on a field that
    starts at exactly 0 its decision follows the sign of FFT round-off; starting one
    sample later makes the decision unambiguous for every implementation."""
    T = n_cycles * 2 * np.pi / omega
    n = int(T / dt) + 1
    if skip_first:
        n += 1
    if even and (n - (1 if skip_first else 0)) % 2:
        n += 1
    t = dt * np.arange(n) if exact_dt else np.linspace(0.0, T, n)
    if skip_first:
        t = t[1:]
    E = E0 * np.sin(np.pi * t / T) ** 2 * np.cos(omega * t + cep)
    return t, E


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def plateau_error(F_test, F_ref, omega, omega0=OMEGA0, q_lo=11, q_hi=41):
    """Relative L2 error of |F|^2 over the harmonic window [q_lo, q_hi] omega0."""
    sel = (omega >= q_lo * omega0) & (omega <= q_hi * omega0)
    a = np.abs(np.asarray(F_test)[sel]) ** 2
    b = np.abs(np.asarray(F_ref)[sel]) ** 2
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
