"""Far field on the GPU against the reference (golden fixtures from Hankel_transform.py)
and the oracle.

Plain form (FP64, the reference's arithmetic): relative error <= 1e-10 of the largest
value, per output.  Fast form (multiplication theorem, FP32): per-harmonic relative L2
error over rho <= 2e-5 (the stated bound of the chosen form), planes <= 2e-5."""
import ctypes
import glob
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIX = sorted(glob.glob(os.path.join(GOLDEN, "hankel_*.npz")))
FAST_TOL = 2e-5


def per_harmonic(a, b):
    """max over omega of ||a[:, w] - b[:, w]|| / ||b[:, w]|| (arrays [rho, omega])."""
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


def _run(g, form):
    from mma_gb300 import hankel as H

    gas = g["gas"].item().decode() if isinstance(g["gas"].item(), bytes) else str(g["gas"])
    H.XUV_index.set_constant_index(complex(g["n_xuv"][0], g["n_xuv"][1]))
    target = H.FSources_provider(g["zgrid"], g["rgrid"], g["ogrid"], data_source="static", FSource=g["S"])
    vac = gas == "vacuum"
    return H.Hankel_long(target, float(g["distance"]), g["rho"], preset_gas=gas, pressure=1.0,
                         near_field_factor=bool(g["near_field"]), store_cumulative_result="cumulative" in g,
                         include_dispersion=not vac, include_absorption=not vac, form=form)


@pytest.mark.parametrize("path", FIX, ids=[os.path.basename(p)[:-4] for p in FIX])
def test_plain_matches_reference(gpu_lib, path):
    g = np.load(path)
    h = _run(g, "plain")
    for key, attr in (("FF_integrated", "FF_integrated"), ("entry", "entry_plane_transform"),
                      ("exit", "exit_plane_transform")):
        ref = g[key]
        assert np.abs(getattr(h, attr) - ref).max() < 1e-10 * np.abs(ref).max(), key
    if "cumulative" in g:
        assert np.abs(h.cumulative_field - g["cumulative"]).max() < 1e-10 * np.abs(g["cumulative"]).max()


@pytest.mark.parametrize("path", FIX, ids=[os.path.basename(p)[:-4] for p in FIX])
def test_fast_matches_reference(gpu_lib, path):
    g = np.load(path)
    h = _run(g, "fast")
    err = per_harmonic(h.FF_integrated, g["FF_integrated"])
    print(os.path.basename(path), "fast per-harmonic error %.2e, plan %s" % (err, h.fast_plan))
    assert err < FAST_TOL
    assert per_harmonic(h.entry_plane_transform, g["entry"]) < FAST_TOL
    assert per_harmonic(h.exit_plane_transform, g["exit"]) < FAST_TOL


def test_fast_vs_plain_config3_geometry(gpu_lib):
    """Config-3 geometry (D = 1 m, z in [-5, 5] mm, r <= 200 um, rho <= 5 mm, harmonics
    10-42 of 800 nm) at reduced sizes, many planes: fast against plain per harmonic."""
    import sys

    sys.path.insert(0, GOLDEN)
    from make_golden import hankel_inputs
    from mma_gb300 import hankel as H

    H.XUV_index.set_constant_index(complex(1 - 1e-5, 1e-7))
    zgrid, rgrid, ogrid, rho, S = hankel_inputs(24, 256, 64, 96, seed=3)
    res = {}
    for form in ("plain", "fast"):
        t = H.FSources_provider(zgrid, rgrid, ogrid, FSource=S)
        res[form] = H.Hankel_long(t, 1.0, rho, preset_gas="Ar", form=form)
    err = per_harmonic(res["fast"].FF_integrated, res["plain"].FF_integrated)
    print("config-3 geometry fast vs plain per-harmonic error %.2e plan %s" % (err, res["fast"].fast_plan))
    assert err < FAST_TOL
    assert res["fast"].fast_plan["trunc_bound"] < 1e-9


def test_hankel_transform_single_plane(gpu_lib):
    import oracle.hankel as oh
    from mma_gb300 import hankel as H

    rng = np.random.default_rng(5)
    og = np.linspace(1e16, 8e16, 7)
    rg = np.linspace(0, 150e-6, 40)
    rho = np.linspace(0, 4e-3, 21)
    F = (rng.standard_normal((7, 40)) + 1j * rng.standard_normal((7, 40))) * np.exp(-(rg / 60e-6) ** 2)
    pre = np.outer(np.ones(40), np.exp(1j * np.linspace(0, 1, 7)))
    got = H.HankelTransform(og, rg, F, 0.9, rho, pre_factor=pre)
    ref = oh.hankel_plane(og, rg, F, 0.9, rho, pre_row=pre[0])
    assert np.abs(got - ref).max() < 1e-11 * np.abs(ref).max()


def test_radially_modulated_medium(gpu_lib):
    """zr-modulated medium (pre-factor per plane, frequency and radius): plain FP64, the fast form
    and its tensor-core planes against the numpy restatement with the same pre-factor table
    (integrated far field, entry plane, non-normalised cumulative field)."""
    import oracle.hankel as oh
    from mma_gb300 import hankel as H

    g = np.load(os.path.join(GOLDEN, "hankel_config3_slice.npz"))
    p = np.load(os.path.join(GOLDEN, "prefactor_radial.npz"))
    H.XUV_index.set_constant_index(complex(g["n_xuv"][0], g["n_xuv"][1]))
    press = dict(zgrid=p["pressure_zgrid"], rgrid=p["pressure_rgrid"], value=p["pressure_value"])
    target = H.FSources_provider(g["zgrid"], g["rgrid"], g["ogrid"], data_source="static", FSource=g["S"])
    ref = oh.hankel_long(g["zgrid"], g["rgrid"], g["ogrid"], g["S"][:-1].astype(np.complex128), float(g["distance"]),
                         g["rho"], cumulative=True, pre=p["pre"])
    for form in ("plain", "fast"):
        h = H.Hankel_long(target, float(g["distance"]), g["rho"], preset_gas="Ar", pressure=press,
                          store_non_normalised_cumulative_result=True, form=form)
        if form == "plain":
            scale = np.abs(ref["FF_integrated"]).max()
            assert np.abs(h.FF_integrated - ref["FF_integrated"]).max() < 1e-10 * scale
            assert np.abs(h.cumulative_field_no_norm - ref["cumulative"]).max() < 1e-10 * scale
        else:
            assert h.fast_plan["planes_via"] == "tc"
            assert per_harmonic(h.FF_integrated, ref["FF_integrated"]) < FAST_TOL
            assert per_harmonic(h.entry_plane_transform, ref["entry"]) < FAST_TOL
            for k in range(ref["cumulative"].shape[0]):
                assert per_harmonic(h.cumulative_field_no_norm[k], ref["cumulative"][k]) < FAST_TOL, k


@pytest.mark.parametrize("n_r,source", [(200, "c64"), (201, "c128")], ids=["even r, complex64", "odd r, complex128"])
def test_series_planes_match_direct_planes(gpu_lib, n_r, source):
    """Up to two requested planes (the entry and exit planes) come out of the fast form's series
    stage, from the same K_m(y) as the far field; three or more go through one FP32 J0 per term.
    Both evaluate J0(k r rho / D_k): per-harmonic agreement within 1e-6, and the far field itself is
    bit-identical whichever way the planes went (the series adds independent sums only)."""
    from mma_gb300 import hankel as H

    omega0 = 0.057 / 2.4188843265857e-17
    rg = np.linspace(0.0, 200e-6, n_r)
    zg = np.linspace(-5e-3, 5e-3, 30)
    og = np.linspace(10 * omega0, 42 * omega0, 12)
    rho = np.linspace(0.0, 5e-3, 40)
    rng = np.random.default_rng(n_r)
    S = np.exp(-(rg / 50e-6) ** 2)[None, None, :] * np.exp(1j * rng.uniform(0, 6.28, (len(zg), len(og))))[:, :, None]
    S = torch.tensor(S, dtype=torch.complex64 if source == "c64" else torch.complex128, device="cuda")
    pre = np.exp(1j * np.linspace(0, 1, len(zg)))[:, None] * np.ones((1, len(og)))
    ff2, p2, plan2 = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=(0, -1), form="fast",
                                 planes_via="direct")
    ff3, p3, plan3 = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=(0, 7, -1), form="fast",
                                 planes_via="direct")
    assert plan2["planes_via"] == "series" and plan3["planes_via"] == "direct"
    assert torch.equal(ff2, ff3)
    for k in (0, len(zg) - 1):
        assert per_harmonic(p2[k].cpu().numpy(), p3[k].cpu().numpy()) < 1e-6, k
    _, p1, _ = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=(7,), form="fast", planes_via="direct")
    assert per_harmonic(p1[7].cpu().numpy(), p3[7].cpu().numpy()) < 1e-6


@pytest.mark.parametrize("n_r,near", [(512, True), (300, False)], ids=["512 r, near field", "300 r, far only"])
def test_stage1_tensor_cores_match_cuda_cores(gpu_lib, n_r, near):
    """Stage 1 of the fast form on the tensor cores (TF32 split precision, 16 series terms) against
    the CUDA-core ring (FP32 FMAs) on the same complex64 source, and both against the plain FP64
    form: the two forms agree within 2e-5 per harmonic (TF32 split precision) and both stay within
    the fast form's bound against FP64.  300 radii leave a partial CTA block."""
    from mma_gb300 import hankel as H

    omega0 = 0.057 / 2.4188843265857e-17
    rg = np.linspace(0.0, 200e-6, n_r)
    zg = np.linspace(-5e-3, 5e-3, 61)
    og = np.linspace(10 * omega0, 42 * omega0, 12)
    rho = np.linspace(0.0, 5e-3, 48)
    rng = np.random.default_rng(n_r)
    S = np.exp(-(rg / 50e-6) ** 2)[None, None, :] * np.exp(1j * rng.uniform(0, 6.28, (len(zg), len(og))))[:, :, None]
    S = torch.tensor(S, dtype=torch.complex64, device="cuda")
    pre = np.exp(1j * np.linspace(0, 1, len(zg)))[:, None] * np.exp(-0.1j * np.arange(len(og)))[None, :]
    out = {}
    try:
        for form in ("tc", "cuda"):
            H.set_stage1_form(form)
            out[form] = H.far_field(og, rg, zg, rho, S, 1.0, pre, near, planes=(0, -1), form="fast", tol=1e-9)
    finally:
        H.set_stage1_form("cuda")
    assert out["tc"][2]["n_terms"] == 16
    ff64, p64, _ = H.far_field(og, rg, zg, rho, S, 1.0, pre, near, planes=(0, -1), form="plain")
    ff_tc, ff_cc = out["tc"][0].cpu().numpy(), out["cuda"][0].cpu().numpy()
    assert not np.array_equal(ff_tc, ff_cc)  # the two forms really ran
    assert per_harmonic(ff_tc, ff_cc) < 2e-5
    assert per_harmonic(ff_tc, ff64.cpu().numpy()) < FAST_TOL
    for k in (0, len(zg) - 1):
        assert per_harmonic(out["tc"][1][k].cpu().numpy(), p64[k].cpu().numpy()) < FAST_TOL


@pytest.mark.parametrize("n_omega,n_r", [(600, 256), (513, 130)], ids=["600 frequencies", "513 frequencies, odd block"])
def test_streamed_host_source_matches_device_source(gpu_lib, monkeypatch, n_omega, n_r):
    """A pinned host source is uploaded in blocks of STREAM_BLOCK frequencies on a second stream
    while the blocks already on the device are computed; every frequency is independent and all
    blocks share the plan of the whole range, so the far field and the series planes equal the
    one-shot call on the same source on the device, bit for bit.  600 and 513 frequencies leave
    a short last block (88 and 1)."""
    from mma_gb300 import hankel as H

    omega0 = 0.057 / 2.4188843265857e-17
    rg = np.linspace(0.0, 200e-6, n_r)
    zg = np.linspace(-5e-3, 5e-3, 21)
    og = np.linspace(10 * omega0, 42 * omega0, n_omega)
    rho = np.linspace(0.0, 5e-3, 40)
    rng = np.random.default_rng(n_omega)
    S = np.exp(-(rg / 50e-6) ** 2)[None, None, :] * np.exp(1j * rng.uniform(0, 6.28, (len(zg), n_omega)))[:, :, None]
    host = torch.tensor(S, dtype=torch.complex64).pin_memory()
    pre = np.exp(1j * np.linspace(0, 1, len(zg)))[:, None] * np.exp(-0.1j * np.arange(n_omega) / n_omega)[None, :]
    calls = []
    real = H._far_field_streamed
    monkeypatch.setattr(H, "_far_field_streamed", lambda *a, **k: calls.append(1) or real(*a, **k))
    ff_h, pl_h, plan_h = H.far_field(og, rg, zg, rho, host, 1.0, pre, True, planes=(0, -1), form="fast")
    assert calls, "the streamed path did not run"
    ff_d, pl_d, plan_d = H.far_field(og, rg, zg, rho, host.cuda(), 1.0, pre, True, planes=(0, -1), form="fast")
    torch.cuda.synchronize()
    assert plan_h["n_terms"] == plan_d["n_terms"]
    assert torch.equal(ff_h, ff_d)
    assert sorted(pl_h) == sorted(pl_d)
    for k in pl_d:
        assert torch.equal(pl_h[k], pl_d[k])


def test_ring_bounded_waits_run_out(gpu_lib):
    """With the ring's copies switched off (the test switch of stage 1's bounded waits), every wait
    runs out after its 2 s limit: the call returns, its far field is NaN (the loud failure), and
    the next call in the same context gives the normal result bit for bit."""
    from mma_gb300 import hankel as H

    lib = gpu_lib
    lib.mma_hankel_test_ring_timeout.argtypes = [ctypes.c_int]
    lib.mma_hankel_test_ring_timeout.restype = ctypes.c_int
    omega0 = 0.057 / 2.4188843265857e-17
    rg = np.linspace(0.0, 200e-6, 256)
    zg = np.linspace(-5e-3, 5e-3, 9)
    og = np.linspace(10 * omega0, 42 * omega0, 3)
    rho = np.linspace(0.0, 5e-3, 16)
    rng = np.random.default_rng(11)
    S = np.exp(-(rg / 50e-6) ** 2)[None, None, :] * np.exp(1j * rng.uniform(0, 6.28, (len(zg), len(og))))[:, :, None]
    S = torch.tensor(S, dtype=torch.complex64, device="cuda")
    ref, _, _ = H.far_field(og, rg, zg, rho, S, 1.0, None, True, form="fast")
    assert torch.isfinite(ref).all()
    assert lib.mma_hankel_test_ring_timeout(1) == 0
    try:
        bad, _, _ = H.far_field(og, rg, zg, rho, S, 1.0, None, True, form="fast")
        torch.cuda.synchronize()
    finally:
        lib.mma_hankel_test_ring_timeout(0)
    assert torch.isnan(bad).all()
    good, _, _ = H.far_field(og, rg, zg, rho, S, 1.0, None, True, form="fast")
    torch.cuda.synchronize()
    assert torch.equal(good, ref)


def test_far_field_plan_replays_the_call(gpu_lib):
    """FarFieldPlan records the fast form once as a CUDA graph: a replay gives the far_field call's
    far field and planes bit for bit, and after a new source is copied into the plan's source a
    replay gives the call on that source."""
    from mma_gb300 import hankel as H

    omega0 = 0.057 / 2.4188843265857e-17
    rg = np.linspace(0.0, 200e-6, 256)
    zg = np.linspace(-5e-3, 5e-3, 17)
    og = np.linspace(10 * omega0, 42 * omega0, 40)
    rho = np.linspace(0.0, 5e-3, 32)
    rng = np.random.default_rng(5)

    def source():
        S = np.exp(-(rg / 50e-6) ** 2)[None, None, :] * np.exp(1j * rng.uniform(0, 6.28, (len(zg), len(og))))[:, :, None]
        return torch.tensor(S, dtype=torch.complex64, device="cuda")

    pre = torch.tensor(np.exp(1j * np.linspace(0, 1, len(zg)))[:, None] * np.exp(-0.1j * np.arange(len(og)))[None, :],
                       dtype=torch.complex128, device="cuda")
    S = source()
    plan = H.FarFieldPlan(og, rg, zg, rho, S, 1.0, pre, True, planes=(0, -1))
    ff, pl = plan.replay()
    ref, ref_pl, _ = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=(0, -1), form="fast")
    torch.cuda.synchronize()
    assert torch.equal(ff, ref)
    for k in ref_pl:
        assert torch.equal(pl[k], ref_pl[k])
    S.copy_(source())
    ff2, _ = plan.replay()
    ref2, _, _ = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=(0, -1), form="fast")
    torch.cuda.synchronize()
    assert not torch.equal(ref2, ref)
    assert torch.equal(ff2, ref2)
