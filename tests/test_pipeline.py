"""Microscopic-to-far-field on the GPU (TDSE spectra -> far field without leaving the device).

CPU: the harmonic-window selection against the linear form of the reference's FindInterval
(shared_python/mynumerics.py:58-60) and the SI conversion of omega.
GPU: the fused path against the oracle composition -- the C restatement of the TDSE per
instance, its spectra arranged as FSourceTerm[kz, kr, omega] (merge.py:98-106), the window and
provider slicing of the far-field driver, and the numpy restatement of Hankel_long -- in FP64
(plain forms): relative error <= 1e-8 of the largest far-field value.
"""
import numpy as np
import pytest
import torch

from tests.tdse_cases import A_CONFIG, sin2_pulse


def _find_interval_linear(x, x0):
    n = len(x)
    if x0 > x[-1] or x0 < x[0]:
        raise LookupError
    for k in range(n - 2):
        if x[k] <= x0 < x[k + 1]:
            return k
    return n - 2


def test_find_interval_matches_linear_form():
    from mma_gb300.pipeline import find_interval

    rng = np.random.default_rng(0)
    for _ in range(200):
        x = np.sort(rng.uniform(0, 50, rng.integers(2, 40)))
        for x0 in list(rng.uniform(x[0], x[-1], 10)) + [x[0], x[-1]] + list(x):
            assert find_interval(x, x0) == _find_interval_linear(x, x0)
        with pytest.raises(LookupError):
            find_interval(x, x[-1] + 1.0)


def test_time_unit():
    from mma_gb300.pipeline import OMEGA_AU2SI, TIME_AU

    assert abs(TIME_AU / 2.4188843265857e-17 - 1.0) < 1e-8
    assert abs(OMEGA_AU2SI * TIME_AU - 1.0) < 1e-15


@pytest.mark.gpu
def test_fused_path_matches_oracle_composition(gpu_lib, oracle_built):
    import oracle.hankel as oh
    import oracle.tdse as ot
    from mma_gb300 import hankel as H
    from mma_gb300.pipeline import OMEGA_AU2SI, harmonic_window, microscopic_to_far_field
    from mma_gb300.tdse_batch import TDSEGrids

    num_r, dx = 600, 0.4
    n_r, n_z = 3, 4
    rgrid = np.linspace(0.0, 60e-6, n_r)
    zgrid = np.linspace(-1e-3, 1e-3, n_z)
    t, base = sin2_pulse(2, E0=1.0, skip_first=True)
    dtf = t[1] - t[0]
    amp = np.array([[0.07 * np.exp(-(r / 50e-6) ** 2) * (1.0 - 0.1 * kz) for r in rgrid] for kz in range(n_z)])
    fields = np.stack([amp[kz, kr] * base for kz in range(n_z) for kr in range(n_r)])  # n = kr + kz n_r
    rho = np.linspace(0.0, 2e-3, 16)
    n_xuv = 1.0 - 1e-5 + 1e-7j
    H.XUV_index.set_constant_index(n_xuv)
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=A_CONFIG)], dt=dtf)
    hr = (3.0, 15.0)
    res, far = microscopic_to_far_field(grids, torch.tensor(fields, device="cuda"), dtf, rgrid, zgrid, 0.057, hr,
                                        rho, 1.0, precision="fp64", tmax=t[-1] - t[0], preset_gas="Ar",
                                        form="plain")
    # oracle composition
    x, psi0, _, _ = ot.ground_state(num_r, dx, A_CONFIG, -1.0, 1e-15)
    spec = []
    om = None
    for n in range(n_r * n_z):
        o = ot.propagate(x, psi0, t, fields[n], dx, A_CONFIG)
        spec.append(o["Fsourceterm"])
        om = o["omegagrid"]
    F = np.stack(spec).reshape(n_z, n_r, -1)  # FSourceTerm[kz, kr, omega]
    ko_min, ko_max = harmonic_window(om, 0.057, hr)
    S = F[:, :, ko_min:ko_max].transpose(0, 2, 1)  # [kz, omega, r]
    og_si = OMEGA_AU2SI * om[ko_min:ko_max]
    disp, absorb = oh.constant_index_factors(og_si, n_xuv)
    ref = oh.hankel_long(zgrid, rgrid, og_si, S, 1.0, rho, disp=disp, absorb=absorb)
    got = far.FF_integrated
    assert got.shape == ref["FF_integrated"].shape
    assert np.abs(got - ref["FF_integrated"]).max() < 1e-8 * np.abs(ref["FF_integrated"]).max()
