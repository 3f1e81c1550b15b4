"""The batching form: an uneven batch (different grids, pulse lengths, field strengths)
in persistent launches from the device work queue, replayed as a CUDA graph."""
import numpy as np
import pytest
import torch

from tests.tdse_cases import A_CONFIG, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-8


def _uneven(seed=1, n_inst=7):
    rng = np.random.default_rng(seed)
    half = rng.uniform(40, 160, n_inst)  # x half-width (a.u.)
    params = [dict(num_r=int(round(2 * w / 0.4)), dx=0.4, trg_a=A_CONFIG) for w in half]
    fields, ts = [], []
    for i in range(n_inst):
        nc = int(rng.integers(1, 3))
        T = nc * 2 * np.pi / 0.057
        n = int(T / 0.25)
        n += n % 2
        t = 0.25 * np.arange(1, n + 1)
        E0 = np.exp(rng.uniform(np.log(0.02), np.log(0.075)))
        fields.append(E0 * np.sin(np.pi * t / T) ** 2 * np.cos(0.057 * t + rng.uniform(0, 2 * np.pi)))
        ts.append(t)
    return params, fields, ts


def test_uneven_batch_graph_replay_matches_oracle(gpu_lib, oracle_built):
    import oracle.tdse as ot
    from mma_gb300.tdse_batch import TDSEBatchPlan, TDSEGrids

    params, fields, ts = _uneven()
    grids = TDSEGrids(params, dt=0.25)
    plan = TDSEBatchPlan(grids, [len(f) for f in fields], 0.25, grid_ids=np.arange(len(params)))
    plan.load_fields([torch.tensor(f, device="cuda") for f in fields])
    plan.capture()
    plan.outputs.zero_()
    plan.replay()
    torch.cuda.synchronize()
    res = plan.result()
    for i, p in enumerate(params):
        x, psi0, e, _ = ot.ground_state(p["num_r"], p["dx"], p["trg_a"], -1.0, 1e-15)
        o = ot.propagate(x, psi0, ts[i], fields[i], p["dx"], p["trg_a"])
        s = res.series(i)
        for k in ("sourceterm", "PopTot", "PopInt", "expval"):
            assert rel_l2(s[k].cpu().numpy(), o[k]) < TOL, (i, k)
        assert rel_l2(res.spectrum(i).cpu().numpy(), o["Fsourceterm"]) < TOL
    # replay on new fields: scaled copies give the oracle's scaled-field results
    plan.load_fields([torch.tensor(0.5 * f, device="cuda") for f in fields])
    plan.replay()
    torch.cuda.synchronize()
    p = params[0]
    x, psi0, e, _ = ot.ground_state(p["num_r"], p["dx"], p["trg_a"], -1.0, 1e-15)
    o = ot.propagate(x, psi0, ts[0], 0.5 * fields[0], p["dx"], p["trg_a"])
    assert rel_l2(plan.result().series(0)["sourceterm"].cpu().numpy(), o["sourceterm"]) < TOL


def test_uneven_batch_c64_mixed_table_widths(gpu_lib, oracle_built):
    """Complex64 form over grids of different widths (several kernel shapes in one plan)."""
    import oracle.tdse as ot
    from mma_gb300.tdse_batch import TDSEBatchPlan, TDSEGrids
    from tests.tdse_cases import plateau_error

    rng = np.random.default_rng(4)
    params = [dict(num_r=n, dx=0.1, trg_a=A_CONFIG) for n in (3000, 6000, 9000, 12000)]
    grids = TDSEGrids(params, dt=0.25, c64=True)
    assert sorted(set(grids.m32)) == [16, 24, 40, 48]
    T = 2 * 2 * np.pi / 0.057
    n = int(T / 0.25)
    n += n % 2
    t = 0.25 * np.arange(1, n + 1)
    E = [0.05 * np.sin(np.pi * t / T) ** 2 * np.cos(0.057 * t + rng.uniform(0, 6)) for _ in params]
    plan = TDSEBatchPlan(grids, [n] * 4, 0.25, grid_ids=np.arange(4), precision="c64")
    plan.load_fields([torch.tensor(e, device="cuda") for e in E])
    plan.launch()
    torch.cuda.synchronize()
    res = plan.result()
    for i, p in enumerate(params):
        x, psi0, e, _ = ot.ground_state(p["num_r"], p["dx"], p["trg_a"], -1.0, 1e-15)
        o = ot.propagate(x, psi0, t, E[i], p["dx"], p["trg_a"])
        err = plateau_error(res.spectrum(i).cpu().numpy(), o["Fsourceterm"], o["omegagrid"])
        pt = rel_l2(res.series(i)["PopTot"].cpu().numpy(), o["PopTot"])
        print("c64 num_r=%d plateau %.2e PopTot %.2e" % (p["num_r"], err, pt))
        assert err < 1e-3 and pt < 2e-4
