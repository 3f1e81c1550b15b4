"""TDSE analysis functions: photoelectron spectrum (window_analysis) and Gabor transform.

CPU: the numpy restatement (oracle/analysis.py) against the reference DLL's own outputs
(tests/golden/analysis.npz, made by tests/golden/make_golden.py from window_analysis and
GaborTransform of the reference built from its sources).
GPU: the library's legacy symbols through TDSE_DLL (the reference's host calls) against the same
fixture, and the batched device API against the oracle on other sizes; FP64 throughout,
relative error <= 1e-9 of the largest value.
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "analysis.npz")
TOL = 1e-9


def _fix():
    return np.load(GOLDEN)


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def test_oracle_pes_matches_reference():
    import oracle.analysis as oa

    g = _fix()
    E0, nE, eps, Es = g["pes_kw"]
    P = oa.pes(g["psi"], int(g["num_r"]), float(g["dx"]), float(g["trg_a"]), int(nE), eps, Es, E0)
    assert _rel(P, g["PES"]) < 1e-11


def test_oracle_gabor_matches_reference():
    import oracle.analysis as oa

    g = _fix()
    om, t0, t1, NG, a = g["gab_kw"]
    G = oa.gabor(g["signal"], float(g["dt"]), int(g["N"]), g["omegas"].size, int(NG), t0, t1, a)
    assert _rel(G.T, g["gabor"]) < 1e-12


@pytest.mark.gpu
def test_legacy_symbols_match_reference(gpu_lib):
    from mma_gb300.structures import inputs_def
    from mma_gb300.tdse import TDSE_DLL

    g = _fix()
    dll = TDSE_DLL()
    inp = inputs_def()
    inp.init_default_inputs(num_r=int(g["num_r"]), dx=float(g["dx"]), trg_a=float(g["trg_a"]))
    E0, nE, eps, Es = g["pes_kw"]
    E, P = dll.compute_PES(inp, g["psi"], E_start=E0, num_E=int(nE), epsilon=eps, Estep=Es)
    assert np.allclose(E, g["E"]) and _rel(P, g["PES"]) < TOL
    om, t0, t1, NG, a = g["gab_kw"]
    tg, omg, G = dll.gabor_transform(g["signal"], float(g["dt"]), int(g["N"]), om, t0, t1, int(NG), a)
    assert np.array_equal(omg, g["omegas"]) and G.shape == g["gabor"].shape
    assert _rel(G, g["gabor"]) < TOL


@pytest.mark.gpu
def test_batched_pes_vs_oracle(gpu_lib):
    import torch

    import oracle.analysis as oa
    from mma_gb300 import analysis

    rng = np.random.default_rng(4)
    num_r, dx, a = 1200, 0.25, 1.0
    x = np.arange(num_r + 1) * dx - 0.5 * num_r * dx
    psi = np.exp(-((x - 10) / 8) ** 2) * np.exp(1j * 0.6 * x) + 0.1 * rng.standard_normal(x.size)
    # chunk smaller than num_E: several launches, each with its own energies
    E, P = analysis.pes(torch.tensor(psi, device="cuda"), num_r, dx, a, E_start=-0.3, num_E=333, epsilon=4e-3,
                        Estep=3e-3, chunk=100)
    ref = oa.pes(psi, num_r, dx, a, 333, 4e-3, 3e-3, -0.3)
    assert _rel(P.cpu().numpy(), ref) < TOL


@pytest.mark.gpu
def test_batched_gabor_vs_oracle(gpu_lib):
    import torch

    import oracle.analysis as oa
    from mma_gb300 import analysis

    rng = np.random.default_rng(5)
    n_sig, N, dt = 5, 1001, 0.3  # odd length: the DFT of the reference's arbitrary N
    t = dt * np.arange(N)
    sig = np.stack([np.cos((0.05 + 0.01 * s) * t) * np.exp(-((t - 150) / 60) ** 2) + 0.01 * rng.standard_normal(N)
                    for s in range(n_sig)])
    tg, om, G = analysis.gabor(torch.tensor(sig, device="cuda"), dt, 2.0, 10.0, 290.0, 40, a=6.0)
    Gh = G.cpu().numpy()
    for s in range(n_sig):
        ref = oa.gabor(sig[s], dt, N, len(om), 40, 10.0, 290.0, 6.0)
        assert _rel(Gh[s], ref) < TOL, s
