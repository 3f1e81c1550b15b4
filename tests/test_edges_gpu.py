"""Edge sizes of the batched GPU entry points against the oracle: the smallest shapes each kernel
accepts, a single instance, a single frequency / radius / screen point, and a single energy or
window.  Tolerances are the forms' own: FP64 plain forms relative error <= 1e-8 (TDSE, relative
L2) and <= 1e-10 of the largest value (far field); fast far field per-harmonic <= 2e-5; analysis
functions <= 1e-9 of the largest value.
"""
import numpy as np
import pytest
import torch

from tests.tdse_cases import A_CONFIG, rel_l2, sin2_pulse

pytestmark = pytest.mark.gpu


def test_tdse_single_instance_tiny_grid(gpu_lib, oracle_built):
    """One instance on a 65-site grid (one site per thread) with a 40-sample field."""
    import oracle.tdse as ot
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    num_r, dx = 64, 0.4
    t = 0.25 * np.arange(1, 41)
    E = 0.05 * np.sin(np.pi * t / (t[-1] + 0.25)) ** 2 * np.cos(0.3 * t)
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=A_CONFIG)], dt=0.25)
    res = run_batch(grids, torch.tensor(E[None, :], device="cuda"), dt_field=0.25, tmax=t[-1] - t[0])
    torch.cuda.synchronize()
    x, psi0, e, _ = ot.ground_state(num_r, dx, A_CONFIG, -1.0, 1e-15)
    o = ot.propagate(x, psi0, t, E, dx, A_CONFIG)
    # the inverse iteration stops on |dE| <= CV in both; on a grid this small the two summation
    # orders leave the energies 1e-11 apart, rounding of an iteration stopped by a tolerance
    assert abs(grids.Einit[0] - e) < 1e-10 * abs(e)
    for k in ("sourceterm", "PopTot", "PopInt", "expval"):
        assert rel_l2(res[k][0].cpu().numpy(), o[k]) < 1e-8, k


def test_far_field_single_frequency_radius_and_screen_point(gpu_lib, oracle_built):
    """One frequency, two radii (the trapezoid's minimum), one screen radius, two planes."""
    import oracle.hankel as oh
    from mma_gb300 import hankel as H

    omega0 = 0.057 / 2.4188843265857e-17
    ogrid = np.array([21 * omega0])
    rgrid = np.array([0.0, 40e-6])
    zgrid = np.array([-1e-3, 0.0, 1e-3])
    rho = np.array([1.5e-3])
    S = (np.array([[[1.0 + 0.5j, 0.25 - 0.1j]], [[0.8 - 0.2j, 0.3 + 0.2j]], [[0.0, 0.0]]]))  # [kz, omega, r]
    n_xuv = complex(1 - 1e-5, 1e-7)
    H.XUV_index.set_constant_index(n_xuv)
    disp, absorb = oh.constant_index_factors(ogrid, n_xuv)
    ref = oh.hankel_long(zgrid, rgrid, ogrid, S, 1.0, rho, disp=disp, absorb=absorb)
    for form in ("plain", "fast"):
        target = H.FSources_provider(zgrid, rgrid, ogrid, data_source="static", FSource=S)
        h = H.Hankel_long(target, 1.0, rho, preset_gas="Ar", form=form)
        got, want = np.asarray(h.FF_integrated), ref["FF_integrated"]
        assert got.shape == want.shape == (1, 1)
        tol = 1e-10 if form == "plain" else 2e-5
        assert np.abs(got - want).max() <= tol * np.abs(want).max(), form
        assert np.abs(np.asarray(h.entry_plane_transform) - ref["entry"]).max() <= tol * np.abs(ref["entry"]).max()


def test_single_energy_and_single_window(gpu_lib):
    """The photoelectron spectrum at one energy and the Gabor transform with one window."""
    import oracle.analysis as oa
    from mma_gb300 import analysis

    num_r, dx, a = 300, 0.4, 1.0
    x = np.arange(num_r + 1) * dx - 0.5 * num_r * dx
    psi = np.exp(-((x - 5) / 6) ** 2) * np.exp(0.4j * x)
    _, P = analysis.pes(torch.tensor(psi, device="cuda"), num_r, dx, a, E_start=0.05, num_E=1, epsilon=4e-3,
                        Estep=3e-3)
    ref = oa.pes(psi, num_r, dx, a, 1, 4e-3, 3e-3, 0.05)
    assert P.shape[0] == 1 and abs(P.cpu().numpy()[0] - ref[0]) <= 1e-9 * abs(ref[0])
    t = 0.3 * np.arange(400)
    sig = np.cos(0.2 * t) * np.exp(-((t - 60) / 30) ** 2)
    _, om, G = analysis.gabor(torch.tensor(sig[None, :], device="cuda"), 0.3, 1.0, 0.0, 100.0, 1, a=5.0)
    refg = oa.gabor(sig, 0.3, len(t), len(om), 1, 0.0, 100.0, 5.0)
    Gh = G.cpu().numpy()[0]
    assert Gh.shape == refg.shape and np.abs(Gh - refg).max() <= 1e-9 * np.abs(refg).max()


def test_df64_one_site_per_thread(gpu_lib, oracle_built):
    """The float-float form on a 65-site grid: one site per thread, so each pass's operand ring
    holds a single site (the prologue copies one, the rest of the ring stays empty)."""
    import oracle.tdse as ot
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    num_r, dx = 64, 0.4
    t = 0.25 * np.arange(1, 41)
    E = 0.05 * np.sin(np.pi * t / (t[-1] + 0.25)) ** 2 * np.cos(0.3 * t)
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=A_CONFIG)], dt=0.25, df64=True)
    res = run_batch(grids, torch.tensor(E[None, :], device="cuda"), dt_field=0.25, tmax=t[-1] - t[0],
                    precision="df64")
    torch.cuda.synchronize()
    x, psi0, e, _ = ot.ground_state(num_r, dx, A_CONFIG, -1.0, 1e-15)
    o = ot.propagate(x, psi0, t, E, dx, A_CONFIG)
    for k in ("sourceterm", "PopTot", "PopInt", "expval"):
        assert rel_l2(res[k][0].cpu().numpy(), o[k]) < 1e-9, k


def test_tensor_core_planes_one_k_block(gpu_lib):
    """Every plane on the tensor cores with 20 radii: one K-block per tile, so most generator
    groups have no K-block in a tile and only run their share of the epilogue."""
    from mma_gb300 import hankel as H

    omega0 = 0.057 / 2.4188843265857e-17
    rg = np.linspace(0.0, 100e-6, 20)
    zg = np.linspace(-5e-3, 5e-3, 24)
    og = np.linspace(10 * omega0, 42 * omega0, 12)
    rho = np.linspace(0.0, 4e-3, 30)
    rng = np.random.default_rng(1)
    S = np.exp(-(rg / 40e-6) ** 2)[None, None, :] * np.exp(1j * rng.uniform(0, 2 * np.pi, (len(zg), len(og))))[:, :, None]
    S = torch.tensor(S, dtype=torch.complex64, device="cuda")
    planes = list(range(len(zg)))
    _, p64, _ = H.far_field(og, rg, zg, rho, S, 1.0, None, True, planes=planes, form="plain")
    _, ptc, plan = H.far_field(og, rg, zg, rho, S, 1.0, None, True, planes=planes, form="fast", planes_via="tc")
    assert plan["planes_via"] == "tc"
    for k in planes:
        a, b = ptc[k].cpu().numpy(), p64[k].cpu().numpy()
        err = (np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)).max()
        assert err < 2e-5, (k, err)


def test_host_tensors_are_moved_to_the_gpu(gpu_lib):
    """Host tensors passed to the tensor-level entry points are copied to the GPU (the kernels take
    device pointers only) and give the same results as device tensors."""
    from mma_gb300 import analysis
    from mma_gb300 import hankel as H

    num_r, dx, a = 200, 0.4, 1.0
    x = np.arange(num_r + 1) * dx - 0.5 * num_r * dx
    psi = torch.tensor(np.exp(-((x - 3) / 5) ** 2) * np.exp(0.3j * x))
    _, Pd = analysis.pes(psi.cuda(), num_r, dx, a, E_start=0.05, num_E=64, epsilon=4e-3, Estep=3e-3)
    _, Ph = analysis.pes(psi, num_r, dx, a, E_start=0.05, num_E=64, epsilon=4e-3, Estep=3e-3)
    assert Ph.is_cuda and torch.equal(Ph, Pd)
    sig = torch.tensor(np.cos(0.2 * 0.3 * np.arange(300))[None, :])
    Gd = analysis.gabor(sig.cuda(), 0.3, 1.0, 0.0, 80.0, 4)[2]
    Gh = analysis.gabor(sig, 0.3, 1.0, 0.0, 80.0, 4)[2]
    assert Gh.is_cuda and torch.equal(Gh, Gd)
    omega0 = 0.057 / 2.4188843265857e-17
    rg, zg = np.linspace(0.0, 60e-6, 16), np.linspace(-1e-3, 1e-3, 5)
    og, rho = np.array([15 * omega0, 21 * omega0]), np.linspace(0.0, 2e-3, 8)
    S = torch.tensor(np.exp(-(rg / 30e-6) ** 2)[None, None, :] * np.ones((len(zg), len(og), 1)), dtype=torch.complex64)
    ffd = H.far_field(og, rg, zg, rho, S.cuda(), 1.0, None, True, form="fast")[0]
    ffh = H.far_field(og, rg, zg, rho, S, 1.0, None, True, form="fast")[0]
    assert ffh.is_cuda and torch.equal(ffh, ffd)
