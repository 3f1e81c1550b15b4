"""Tabulated XUV refractive index (XUV_index.load_tables) against the reference's own module.

The fixture tests/golden/xuv_index.npz holds dispersion_function and beta_factor_ref of
shared_python/XUV_refractive_index.py, fed by shared_python/make_table.py, both run unchanged on
the synthetic tables in tests/golden/xuv_tables (see tests/golden/make_golden.py).  The provider
reads the same text tables directly.
"""
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture()
def tables():
    from mma_gb300 import hankel as H

    H.XUV_index.load_tables(os.path.join(HERE, "xuv_tables"))
    yield H
    H.XUV_index.set_constant_index(complex(1 - 1e-5, 1e-7))


def test_provider_matches_reference_module(tables):
    H = tables
    g = np.load(os.path.join(HERE, "xuv_index.npz"))
    assert sorted(H.XUV_index.gases) == sorted(g["gases"].tolist())
    for gas in g["gases"]:
        d = H.XUV_index.dispersion_function(g["omega"], 0.7, str(gas), n_IR=1.0003)
        b = H.XUV_index.beta_factor_ref(g["omega"], str(gas))
        assert np.allclose(d, g["disp_" + gas], rtol=1e-12, atol=0), gas
        assert np.allclose(b, g["beta_" + gas], rtol=1e-12, atol=0), gas


def test_unlisted_and_out_of_range_energies_raise(tables):
    H = tables
    ev = 1.602176565e-19 / 1.0545718e-34
    with pytest.raises(ValueError):  # f1 = -9999 (not listed) below 18 eV in the Henke tables
        H.XUV_index.dispersion_function(np.array([12.0 * ev]), 1.0, "Ar_Henke")
    with pytest.raises(ValueError):  # beyond the table
        H.XUV_index.beta_factor_ref(np.array([500.0 * ev]), "Ar_NIST")


def test_pre_factor_uses_tables(tables):
    """The no-modulation pre-factor (Hankel_transform.py:405-448) with a tabulated medium."""
    H = tables
    ev = 1.602176565e-19 / 1.0545718e-34
    w = np.linspace(30.0, 60.0, 5) * ev
    z = np.linspace(-1e-3, 1e-3, 4)
    pre, renorm = H.pre_factor_table(z, w, "Ar", 0.5, "Henke", True, "NIST", True, 1.0)
    disp = 1j * H.XUV_index.dispersion_function(w, 0.5, "Ar_NIST")
    absorb = (0.5 / H.C_LIGHT) * H.XUV_index.beta_factor_ref(w, "Ar_Henke")
    ref = 0.5 * np.exp(w[None, :] * (z[:, None] * disp[None, :] + (z[:, None] - z[-1]) * absorb[None, :]))
    assert np.allclose(pre, ref, rtol=1e-13, atol=0)
    assert np.all(renorm[-1] == 1.0)
