"""Batched TDSE (one persistent launch, device work queue) against the oracle.

Every instance of a batch must equal the oracle's single-instance result within
the FP64 parity tolerance (relative L2 <= 1e-8)."""
import numpy as np
import pytest
import torch

from tests.tdse_cases import A_CONFIG, rel_l2, sin2_pulse

pytestmark = pytest.mark.gpu
TOL = 1e-8


def _oracle(t, E, num_r, dx, a):
    import oracle.tdse as ot

    x, psi0, e, _ = ot.ground_state(num_r, dx, a, -1.0, 1e-15)
    return ot.propagate(x, psi0, t, E, dx, a), e, psi0


def test_batch_uniform_matches_oracle(gpu_lib, oracle_built):
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    t, _ = sin2_pulse(2, skip_first=True)
    rng = np.random.default_rng(7)
    n_inst = 5
    E0 = rng.uniform(0.03, 0.07, n_inst)
    cep = rng.uniform(0, 2 * np.pi, n_inst)
    T = t[-1] + (t[1] - t[0])
    fields = np.stack([e0 * np.sin(np.pi * t / T) ** 2 * np.cos(0.057 * t + c) for e0, c in zip(E0, cep)])
    dtf = t[1] - t[0]
    grids = TDSEGrids([dict(num_r=600, dx=0.4, trg_a=A_CONFIG)], dt=dtf)
    res = run_batch(grids, torch.tensor(fields, device="cuda"), dt_field=dtf, dt_req=0.25,
                    tmax=t[-1] - t[0])
    torch.cuda.synchronize()
    for i in range(n_inst):
        o, e, psi0 = _oracle(t, fields[i], 600, 0.4, A_CONFIG)
        assert abs(grids.Einit[0] - e) < 1e-12
        for k in ("sourceterm", "PopTot", "PopInt", "expval"):
            assert rel_l2(res[k][i].cpu().numpy(), o[k]) < TOL, (i, k)
        assert np.array_equal(res["tgrid"][i].cpu().numpy(), o["tgrid"])
        assert rel_l2(res["Fsourceterm"][i].cpu().numpy(), o["Fsourceterm"]) < TOL


def test_batch_multi_grid_uneven(gpu_lib, oracle_built):
    """Instances on different grids and with different pulse lengths in one launch."""
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    params = [dict(num_r=500, dx=0.4, trg_a=1.0), dict(num_r=900, dx=0.3, trg_a=A_CONFIG),
              dict(num_r=3000, dx=0.1, trg_a=1.2)]
    dtf = 0.25
    grids = TDSEGrids(params, dt=dtf)
    cases = [(0, 1.0), (1, 2.0), (2, 1.5), (1, 1.25), (0, 2.0)]
    fields, ts = [], []
    for g, nc in cases:
        T = nc * 2 * np.pi / 0.057
        n = int(T / dtf)
        n += n % 2
        t = dtf * np.arange(1, n + 1)
        ts.append(t)
        fields.append(0.05 * np.sin(np.pi * t / T) ** 2 * np.cos(0.057 * t))
    res = run_batch(grids, [torch.tensor(f, device="cuda") for f in fields], dt_field=dtf,
                    grid_ids=[c[0] for c in cases], psi_final=True)
    torch.cuda.synchronize()
    for i, (g, _) in enumerate(cases):
        p = params[g]
        o, e, psi0 = _oracle(ts[i], fields[i], p["num_r"], p["dx"], p["trg_a"])
        s = res.series(i)
        for k in ("sourceterm", "PopTot", "PopInt", "expval"):
            assert rel_l2(s[k].cpu().numpy(), o[k]) < TOL, (i, k)
        po = res["psi_off"][i]
        n = p["num_r"] + 1
        psi = res["psi_final"][po:po + 2 * n].cpu().numpy()
        assert rel_l2(psi[0::2] + 1j * psi[1::2], o["psi"]) < TOL


def test_ground_states_match_oracle(gpu_lib, oracle_built):
    from mma_gb300.tdse_batch import TDSEGrids
    import oracle.tdse as ot

    params = [dict(num_r=800, dx=0.25, trg_a=0.8), dict(num_r=8000, dx=0.1, trg_a=A_CONFIG)]
    grids = TDSEGrids(params, dt=0.25)
    for g, p in enumerate(params):
        x, psi0, e, it = ot.ground_state(p["num_r"], p["dx"], p["trg_a"], -1.0, 1e-15)
        assert abs(grids.Einit[g] - e) < 1e-12
        assert np.array_equal(grids.x(g).cpu().numpy(), x)
        assert rel_l2(grids.psi0(g).cpu().numpy(), psi0) < 1e-9
    assert abs(grids.Einit[1] - (-0.538491475066)) < 1e-11
