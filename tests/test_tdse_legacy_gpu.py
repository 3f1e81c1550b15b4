"""GPU parity of the legacy TDSE C-ABI (the reference DLL's symbols) against the oracle.

Tolerance: relative L2 <= 1e-8 in FP64 on the dipole acceleration (sourceterm),
populations and <x>, as the path's FP64 parity target states.
"""
import numpy as np
import pytest

from tests.tdse_cases import A_CONFIG, rel_l2, sin2_pulse

pytestmark = pytest.mark.gpu

TOL = 1e-8


@pytest.fixture(scope="module")
def dll(gpu_lib):
    from mma_gb300.tdse import TDSE_DLL

    return TDSE_DLL()


def _oracle_run(t, E, num_r, dx, a, CV=1e-15, **kw):
    import oracle.tdse as ot

    x, psi0, e, it = ot.ground_state(num_r, dx, a, -1.0, CV)
    o = ot.propagate(x, psi0, t, E, dx, a, **kw)
    o.update(x=x, psi0=psi0, Einit=e)
    return o


@pytest.mark.parametrize("num_r,dx,ncyc", [(600, 0.4, 2), (2000, 0.2, 3)])
def test_legacy_matches_oracle(dll, oracle_built, num_r, dx, ncyc):
    from mma_gb300.tdse import run_single

    t, E = sin2_pulse(ncyc)
    g = run_single(dll, t, E, num_r=num_r, dx=dx, trg_a=A_CONFIG, CV=1e-15)
    o = _oracle_run(t, E, num_r, dx, A_CONFIG)
    assert abs(g["Einit"] - o["Einit"]) < 1e-12
    assert rel_l2(np.abs(g["psi0"]), np.abs(o["psi0"])) < 1e-10
    assert np.array_equal(g["x"], o["x"])
    assert g["Nt"] == o["n_out"] and g["Nomega"] == o["n_omega"]
    assert np.array_equal(g["tgrid"], o["tgrid"])
    assert np.array_equal(g["Efield"], o["Efield"])  # k1 = 1: both copy the samples exactly
    for k in ("sourceterm", "PopTot", "PopInt", "expval"):
        assert rel_l2(g[k], o[k]) < TOL, k
    assert rel_l2(g["Fsourceterm"], o["Fsourceterm"]) < TOL
    assert rel_l2(g["FsourcetermM2"], o["FsourcetermM2"]) < TOL
    assert rel_l2(g["FEfield"], o["FEfield"]) < 1e-12
    assert np.allclose(g["omegagrid"], o["omegagrid"], rtol=1e-14, atol=0)


def test_legacy_snapshots(dll, oracle_built):
    from mma_gb300.tdse import run_single

    t, E = sin2_pulse(1.5)
    g = run_single(dll, t, E, num_r=600, dx=0.4, trg_a=1.0, CV=1e-15, writewft=1, tprint=10.0)
    o = _oracle_run(t, E, 600, 0.4, 1.0, writewft=1, tprint=10.0)
    assert g["snapshots"].shape == o["snapshots"].shape
    assert rel_l2(g["snapshots"], o["snapshots"]) < TOL
