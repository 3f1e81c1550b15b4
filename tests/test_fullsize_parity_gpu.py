"""Parity at the benchmark's full sizes, on the GPU, against the reference and the oracle.

* config 0 -- one 8001-site instance, 10-cycle 800 nm pulse, 4412 steps -- through the legacy
  C-ABI (the reference DLL's symbols, driven by the same TDSE_DLL host class that drove the
  reference DLL to make tests/golden/tdse_config0.npz) and through the batched entry point in
  the FP64 plain form and the float-float form;
* seeded instances of config 1 (the 64 r x 32 z Gaussian focus, 8001 sites, 4412 steps)
  against the oracle run on the host;
* a field sampled at 0.5 a.u. for dt = 0.25 (Fourier interpolation with k1 = 3, the device
  FFT path and the zero gate on the interpolated field) against the reference's fixture
  tests/golden/tdse_interp.npz, through both entry points.

Tolerances: relative L2 <= 1e-8 (the path's FP64 parity target) on every series and on the
spectrum for both forms against the reference or the oracle; the float-float form also within
1e-9 of the FP64 form on the same instances; Einit within 1e-12 and the x grid bit-identical.

Why the float-float form's bar against the oracle is the FP64 one: the inverse iteration stops
at |dE| <= CV = 1e-15, where the oracle's and the GPU's ground states agree to about 1e-11.  At
the weak-field edge of the focus (peak field ~1.5e-3 a.u.) the dipole acceleration is only a few
per cent of the field, and that residue of excited states shows up in it: a 1.1e-8 change of the
ground state moves such an instance's sourceterm by 1.3e-5 (the oracle alone, CV 1e-15 against
1e-12).  Both GPU forms start from the same GPU ground state, so they agree far more closely with
each other than either does with the oracle there.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest
import torch

from tests.tdse_cases import A_CONFIG, rel_l2

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-8
TOL_DF64 = 1e-9
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SERIES = ("sourceterm", "PopTot", "PopInt", "expval")


def _fixture(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _check_against(res, ref, tol, what):
    errs = {}
    for k in SERIES:
        errs[k] = rel_l2(res[k], ref[k])
    errs["Fsourceterm"] = rel_l2(res["Fsourceterm"], ref["Fsourceterm"])
    print("%s: %s" % (what, ", ".join("%s %.2e" % kv for kv in errs.items())))
    for k, e in errs.items():
        assert e < tol, (what, k, e)


@pytest.fixture(scope="module")
def config0():
    return _fixture("tdse_config0")


def test_config0_legacy_abi_matches_reference_fixture(gpu_lib, config0):
    from mma_gb300.tdse import TDSE_DLL, run_single

    g = config0
    num_r, dx, a = int(g["params"][0]), float(g["params"][1]), float(g["params"][2])
    r = run_single(TDSE_DLL(), g["t"], g["E"], num_r=num_r, dx=dx, trg_a=a, CV=1e-15)
    assert abs(r["Einit"] - float(g["Einit"])) < 1e-12
    assert np.array_equal(r["x"], g["x"])
    assert rel_l2(np.real(r["psi0"]), g["psi0_re"]) < 1e-10
    assert r["Nt"] == int(g["Nt"]) and r["Nomega"] == int(g["Nomega"])
    assert np.array_equal(r["tgrid"], g["tgrid"])
    assert rel_l2(r["Efield"], g["Efield"]) < 1e-13
    _check_against(r, g, TOL_FP64, "config 0, legacy ABI")
    assert rel_l2(r["FsourcetermM2"], g["FsourcetermM2"]) < TOL_FP64
    assert rel_l2(r["FEfield"], g["FEfield"]) < 1e-12
    assert np.allclose(r["omegagrid"], g["omegagrid"], rtol=1e-14, atol=0)


@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("df64", TOL_DF64)])
def test_config0_batch_matches_reference_fixture(gpu_lib, config0, precision, tol):
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    g = config0
    num_r, dx, a = int(g["params"][0]), float(g["params"][1]), float(g["params"][2])
    t = g["t"]
    dtf = float(t[1] - t[0])
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=a)], dt=dtf, df64=(precision == "df64"))
    assert abs(grids.Einit[0] - float(g["Einit"])) < 1e-12
    assert np.array_equal(grids.x(0).cpu().numpy(), g["x"])
    res = run_batch(grids, torch.tensor(g["E"][None, :], device="cuda"), dt_field=dtf,
                    tmax=float(t[-1] - t[0]), precision=precision)
    torch.cuda.synchronize()
    out = {k: res[k][0].cpu().numpy() for k in SERIES + ("tgrid",)}
    out["Fsourceterm"] = res["Fsourceterm"][0].cpu().numpy()
    assert np.array_equal(out["tgrid"], g["tgrid"])
    _check_against(out, g, tol, "config 0, batch %s" % precision)


def _oracle_run(args):
    import oracle.tdse as ot

    t, E, x, psi0 = args
    return ot.propagate(x, psi0, t, E, 0.1, A_CONFIG)


def test_config1_instances_match_oracle(gpu_lib, oracle_built):
    """Eight seeded instances of the config-1 focus (8001 sites, 4412 steps) in one batch, FP64
    and float-float, each against the oracle run on the host (threads; the oracle's C calls
    release the interpreter lock)."""
    import oracle.tdse as ot
    from bench import focus_fields
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    t, fields = focus_fields()
    rng = np.random.default_rng(2024)
    pick = np.sort(rng.choice(fields.shape[0], size=8, replace=False))
    sub = fields[pick]
    dtf = float(t[1] - t[0])
    x, psi0, e, _ = ot.ground_state(8000, 0.1, A_CONFIG, -1.0, 1e-15)
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        refs = list(ex.map(_oracle_run, [(t, sub[i], x, psi0) for i in range(len(pick))]))
    grids = TDSEGrids([dict(num_r=8000, dx=0.1, trg_a=A_CONFIG)], dt=dtf, df64=True)
    assert abs(grids.Einit[0] - e) < 1e-12
    outs = {}
    for precision in ("fp64", "df64"):
        res = run_batch(grids, torch.tensor(sub, device="cuda"), dt_field=dtf, tmax=float(t[-1] - t[0]),
                        precision=precision)
        torch.cuda.synchronize()
        outs[precision] = []
        for i, n in enumerate(pick):
            out = {k: res[k][i].cpu().numpy() for k in SERIES + ("tgrid",)}
            out["Fsourceterm"] = res["Fsourceterm"][i].cpu().numpy()
            assert np.array_equal(out["tgrid"], refs[i]["tgrid"])
            _check_against(out, refs[i], TOL_FP64, "config 1 instance %d, %s" % (n, precision))
            outs[precision].append(out)
    for i, n in enumerate(pick):
        _check_against(outs["df64"][i], outs["fp64"][i], TOL_DF64, "config 1 instance %d, df64 against fp64" % n)


def test_interpolated_field_matches_reference_fixture(gpu_lib):
    """k1 = 3: the field is Fourier-interpolated on the device before propagation."""
    from mma_gb300.tdse import TDSE_DLL, run_single
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    g = _fixture("tdse_interp")
    num_r, dx, a = int(g["params"][0]), float(g["params"][1]), float(g["params"][2])
    t, E = g["t"], g["E"]
    r = run_single(TDSE_DLL(), t, E, num_r=num_r, dx=dx, trg_a=a, dt=0.25, CV=1e-15)
    assert r["Nt"] == int(g["Nt"])
    assert np.array_equal(r["tgrid"], g["tgrid"])
    assert rel_l2(r["Efield"], g["Efield"]) < 1e-12
    _check_against(r, g, TOL_FP64, "k1 = 3, legacy ABI")

    dtf = float(t[1] - t[0])
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=a)], dt=float(g["dt"]))
    res = run_batch(grids, torch.tensor(E[None, :], device="cuda"), dt_field=dtf, dt_req=0.25,
                    tmax=float(t[-1] - t[0]))
    torch.cuda.synchronize()
    assert res["k1"] == 3
    out = {k: res[k][0].cpu().numpy() for k in SERIES + ("tgrid", "Efield")}
    out["Fsourceterm"] = res["Fsourceterm"][0].cpu().numpy()
    assert np.array_equal(out["tgrid"], g["tgrid"])
    assert rel_l2(out["Efield"], g["Efield"]) < 1e-12
    _check_against(out, g, TOL_FP64, "k1 = 3, batch")
