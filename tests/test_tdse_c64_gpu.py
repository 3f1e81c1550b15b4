"""The complex64 form (FP32 propagation, FP64 factorisation and final accumulation)
against the FP64 oracle: its error is measured and bounded, not parity-exact.

Stated bounds (this test's tolerances), 2-cycle 0.0534 a.u. pulses on three grids:
relative L2 of populations and <x> <= 2e-4, of the dipole acceleration (sourceterm,
which nearly cancels E and <V'>) <= 1e-3, plateau |F|^2 (harmonics 11-41) <= 1e-3."""
import numpy as np
import pytest
import torch

from tests.tdse_cases import A_CONFIG, plateau_error, rel_l2, sin2_pulse

pytestmark = pytest.mark.gpu
BOUNDS = {"sourceterm": 1e-3, "PopTot": 2e-4, "PopInt": 2e-4, "expval": 2e-4, "plateau": 1e-3}


def test_c64_against_oracle(gpu_lib, oracle_built):
    import oracle.tdse as ot
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    t, E = sin2_pulse(2, skip_first=True)
    dtf = t[1] - t[0]
    report = {}
    for num_r, dx in [(600, 0.4), (2000, 0.2), (8000, 0.1)]:
        grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=A_CONFIG)], dt=dtf, c64=True)
        f = torch.tensor(np.stack([E, 0.8 * E]), device="cuda")
        r32 = run_batch(grids, f, dt_field=dtf, tmax=t[-1] - t[0], precision="c64")
        torch.cuda.synchronize()
        x, psi0, e, _ = ot.ground_state(num_r, dx, A_CONFIG, -1.0, 1e-15)
        o = ot.propagate(x, psi0, t, E, dx, A_CONFIG)
        errs = {k: rel_l2(r32[k][0].cpu().numpy(), o[k]) for k in ("sourceterm", "PopTot", "PopInt", "expval")}
        errs["plateau"] = plateau_error(r32["Fsourceterm"][0].cpu().numpy(), o["Fsourceterm"], o["omegagrid"])
        assert np.array_equal(r32["tgrid"][0].cpu().numpy(), o["tgrid"])
        report[num_r] = errs
        print("c64 errors vs FP64 oracle (num_r=%d): %s" % (num_r, {k: "%.2e" % v for k, v in errs.items()}))
    for num_r, errs in report.items():
        for k, b in BOUNDS.items():
            assert errs[k] < b, (num_r, k, errs[k])


@pytest.mark.parametrize("threads", [512, 1024])
def test_c64_cta_sizes_against_oracle(gpu_lib, oracle_built, threads):
    """The wider CTA shapes of the complex64 kernel (same tables rounded the same way, wider
    scans): same bounds against the oracle, and close to the 256-thread result."""
    import oracle.tdse as ot
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    t, E = sin2_pulse(2, skip_first=True)
    dtf = t[1] - t[0]
    for num_r, dx in [(600, 0.4), (8000, 0.1)]:
        g_w = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=A_CONFIG)], dt=dtf, c64=True, c64_threads=threads)
        g_n = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=A_CONFIG)], dt=dtf, c64=True)
        assert int(g_w.c64_threads[0]) == threads and int(g_w.m32[0]) * threads >= num_r + 1
        f = torch.tensor(np.stack([E, 0.8 * E]), device="cuda")
        rw = run_batch(g_w, f, dt_field=dtf, tmax=t[-1] - t[0], precision="c64")
        rn = run_batch(g_n, f, dt_field=dtf, tmax=t[-1] - t[0], precision="c64")
        torch.cuda.synchronize()
        x, psi0, e, _ = ot.ground_state(num_r, dx, A_CONFIG, -1.0, 1e-15)
        o = ot.propagate(x, psi0, t, E, dx, A_CONFIG)
        for k in ("sourceterm", "PopTot", "PopInt", "expval"):
            assert rel_l2(rw[k][0].cpu().numpy(), o[k]) < BOUNDS[k], (threads, num_r, k)
            assert rel_l2(rw[k][1].cpu().numpy(), rn[k][1].cpu().numpy()) < BOUNDS[k], (threads, num_r, k)
        assert plateau_error(rw["Fsourceterm"][0].cpu().numpy(), o["Fsourceterm"], o["omegagrid"]) < BOUNDS["plateau"]


def test_c64_mixed_cta_sizes_in_one_plan(gpu_lib):
    """Grids with different CTA sizes in one batch: the plan groups launches by shape."""
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    t, E = sin2_pulse(1, skip_first=True)
    dtf = t[1] - t[0]
    params = [dict(num_r=2000, dx=0.2, trg_a=A_CONFIG), dict(num_r=10000, dx=0.1, trg_a=A_CONFIG)]
    g_mix = TDSEGrids(params, dt=dtf, c64=True, c64_threads=[512, 512])
    assert list(g_mix.c64_threads) == [512, 256]  # 10001 sites do not fit the 512-thread kernel
    g_ref = TDSEGrids(params, dt=dtf, c64=True)
    f = torch.tensor(np.stack([E, E, 0.7 * E]), device="cuda")
    ids = [0, 1, 0]
    rm = run_batch(g_mix, f, dt_field=dtf, grid_ids=ids, precision="c64", tmax=t[-1] - t[0])
    rr = run_batch(g_ref, f, dt_field=dtf, grid_ids=ids, precision="c64", tmax=t[-1] - t[0])
    torch.cuda.synchronize()
    assert torch.isfinite(rm["sourceterm"]).all()
    for i in range(3):
        assert rel_l2(rm["PopTot"][i].cpu().numpy(), rr["PopTot"][i].cpu().numpy()) < 2e-4


def test_autotuner_picks_and_caches(gpu_lib, tmp_path, monkeypatch):
    from mma_gb300 import autotune
    from mma_gb300.tdse_batch import TDSEGrids

    monkeypatch.setenv("MMA_TUNE_CACHE", str(tmp_path / "tune.json"))
    p = dict(num_r=4000, dx=0.1, trg_a=A_CONFIG)
    t = autotune.choose_c64_threads(4001, 0.25, p, retune=True)
    assert t in (256, 512, 1024)
    rep = autotune.last_report()
    key = autotune._key(4001, 0.25, "c64", "cuda")
    assert key in rep and all(v > 0 for v in rep[key].values())
    best = min(rep[key], key=rep[key].get)
    assert t == best or (t == autotune.DEFAULT and rep[key][best] > (1 - autotune.MARGIN) * rep[key][t])
    assert (tmp_path / "tune.json").exists()
    autotune._MEM.clear()
    assert autotune.choose_c64_threads(4001, 0.25, p) == t  # from the file, no timing
    g = TDSEGrids([p], dt=0.25, c64=True, c64_threads="auto")
    assert int(g.c64_threads[0]) == t


def test_c64_default_ctas_follow_occupancy(gpu_lib):
    """Persistent grid of the complex64 form per table shape: two CTAs per SM where the 256-thread
    kernel fits twice (at most 16 sites per thread), one otherwise, none for a shape without a
    kernel."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert gpu_lib.mma_tdse_c64_default_ctas(16, 256) == 2 * sms
    assert gpu_lib.mma_tdse_c64_default_ctas(8, 0) == 2 * sms
    assert gpu_lib.mma_tdse_c64_default_ctas(32, 256) == sms
    assert gpu_lib.mma_tdse_c64_default_ctas(16, 512) == sms
    assert gpu_lib.mma_tdse_c64_default_ctas(12, 256) == 0


def test_c64_uneven_widths_in_one_launch(gpu_lib):
    """Grids of every 256-thread table width (16 to 48 sites per thread: 3001 to 12001 sites) and
    pulses of different lengths in one batch: one launch of the width-dispatching kernel, and the
    same results as one launch per width (the same per-instance code, so equal to FP32 rounding
    of the compiled schedule), all finite."""
    from mma_gb300.tdse_batch import TDSEBatchPlan, TDSEGrids

    params = [dict(num_r=n, dx=0.1, trg_a=A_CONFIG) for n in (3000, 5000, 7000, 9000, 12000)]
    dtf = 0.25
    grids = TDSEGrids(params, dt=dtf, c64=True)
    assert sorted(set(int(m) for m in grids.m32)) == [16, 24, 32, 40, 48]
    rng = np.random.default_rng(3)
    fields, ids = [], []
    for i in range(12):
        T = (1.0 + 0.25 * (i % 4)) * 2 * np.pi / 0.057
        n = int(T / dtf)
        n += n % 2
        t = dtf * np.arange(1, n + 1)
        fields.append(torch.tensor(rng.uniform(0.03, 0.07) * np.sin(np.pi * t / T) ** 2 * np.cos(0.057 * t),
                                   device="cuda"))
        ids.append(i % len(params))
    out = {}
    for one in (True, False):
        plan = TDSEBatchPlan(grids, [len(f) for f in fields], dtf, grid_ids=ids, precision="c64", c64_one_launch=one)
        assert len(plan.launches) == (1 if one else 5)
        plan.load_fields(fields)
        plan.launch()
        torch.cuda.synchronize()
        out[one] = plan
    for i in range(len(fields)):
        a, b = out[True].result().series(i), out[False].result().series(i)
        for k in ("sourceterm", "PopTot", "PopInt", "expval"):
            assert torch.isfinite(a[k]).all()
            assert rel_l2(a[k].cpu().numpy(), b[k].cpu().numpy()) < 1e-6, (i, k)
