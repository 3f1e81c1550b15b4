"""Pin the oracle (the CPU restatement) to the reference itself.

* against the golden fixtures, generated from the reference DLL compiled unchanged
  from its sources (tests/golden/make_golden.py) -- runs everywhere;
* against a live build of that DLL where the reference sources exist (oracle/_ref).
"""
import glob
import os

import numpy as np
import pytest

from tests.tdse_cases import rel_l2, sin2_pulse

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TDSE_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "tdse_*.npz")))


def _oracle_case(g):
    import oracle.tdse as ot

    num_r, dx, a = int(g["params"][0]), float(g["params"][1]), float(g["params"][2])
    x, psi0, e, it = ot.ground_state(num_r, dx, a, -1.0, 1e-15)
    kw = {}
    if "tprint" in g:
        kw = dict(writewft=1, tprint=float(g["tprint"]))
    o = ot.propagate(x, psi0, g["t"], g["E"], dx, a, **kw)
    o.update(x=x, psi0=psi0, Einit=e)
    return o


@pytest.mark.parametrize("path", TDSE_FIXTURES, ids=[os.path.basename(p)[:-4] for p in TDSE_FIXTURES])
def test_oracle_matches_reference_fixture(oracle_built, path):
    g = np.load(path)
    o = _oracle_case(g)
    assert abs(o["Einit"] - float(g["Einit"])) < 1e-13
    assert np.array_equal(o["x"], g["x"])
    assert rel_l2(np.real(o["psi0"]), g["psi0_re"]) < 1e-12
    assert o["n_out"] == int(g["Nt"])
    assert np.array_equal(o["tgrid"], g["tgrid"])
    assert rel_l2(o["Efield"], g["Efield"]) < 1e-13
    for k in ("sourceterm", "PopTot", "PopInt", "expval", "Fsourceterm", "FsourcetermM2", "FEfield"):
        assert rel_l2(o[k], g[k]) < 1e-11, k
    assert np.allclose(o["omegagrid"], g["omegagrid"], rtol=1e-15, atol=0)
    if "snapshots" in g:
        assert rel_l2(o["snapshots"], g["snapshots"]) < 1e-11


def test_oracle_matches_live_reference(oracle_built):
    import oracle

    if oracle.ref_dll_path() is None:
        pytest.skip("reference sources are not present here; the fixtures pin the oracle instead")
    from mma_gb300.tdse import TDSE_DLL, run_single

    dll = TDSE_DLL(oracle.ref_dll_path())
    t, E = sin2_pulse(2.5, E0=0.07, cep=0.4, skip_first=True)
    r = run_single(dll, t, E, num_r=900, dx=0.3, trg_a=1.2, CV=1e-15)
    import oracle.tdse as ot

    x, psi0, e, _ = ot.ground_state(900, 0.3, 1.2, -1.0, 1e-15)
    o = ot.propagate(x, psi0, t, E, 0.3, 1.2)
    assert abs(e - r["Einit"]) < 1e-13
    for k in ("sourceterm", "PopTot", "PopInt", "expval", "Fsourceterm"):
        assert rel_l2(o[k], r[k]) < 1e-11, k


def test_ground_state_known_answer(oracle_built):
    """Survey known answer: a^2 = 1.68, dx = 0.1, num_r = 8000, Eguess = -1, CV = 1e-15."""
    import oracle.tdse as ot

    _, psi0, e, _ = ot.ground_state(8000, 0.1, np.sqrt(1.68), -1.0, 1e-15)
    assert abs(e - (-0.538491475066)) < 1e-11
    assert abs(np.sum(np.abs(psi0) ** 2) - 1.0) < 1e-14


def test_oracle_zero_gate_identity_for_k1_1(oracle_built):
    """A field starting at exactly 0: with k1 = 1 the interpolation is an exact copy and
    the reference's gate (first k with f[k] f[k+1] <= 0) opens at k = 0."""
    import oracle.tdse as ot

    t, E = sin2_pulse(1)
    assert E[0] == 0.0
    x, psi0, e, _ = ot.ground_state(400, 0.4, 1.0, -1.0, 1e-15)
    o = ot.propagate(x, psi0, t, E, 0.4, 1.0)
    assert o["Efield"][1] == 0.0 and o["Efield"][2] == E[1]
