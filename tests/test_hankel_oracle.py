"""Pin the numpy Hankel restatement (oracle/hankel.py) to fixtures generated by the
reference's own Hankel/Hankel_transform.py (tests/golden/make_golden.py)."""
import glob
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIX = sorted(glob.glob(os.path.join(GOLDEN, "hankel_*.npz")))


def oracle_from_fixture(g):
    import oracle.hankel as oh

    gas = g["gas"].item().decode() if isinstance(g["gas"].item(), bytes) else str(g["gas"])
    n = complex(g["n_xuv"][0], g["n_xuv"][1])
    disp = absorb = None
    if gas != "vacuum":
        disp, absorb = oh.constant_index_factors(g["ogrid"], n)
    return oh.hankel_long(g["zgrid"], g["rgrid"], g["ogrid"], g["S"], float(g["distance"]), g["rho"], disp=disp,
                          absorb=absorb, near_field=bool(g["near_field"]), cumulative="cumulative" in g)


@pytest.mark.parametrize("path", FIX, ids=[os.path.basename(p)[:-4] for p in FIX])
def test_hankel_oracle_matches_reference(path):
    g = np.load(path)
    o = oracle_from_fixture(g)
    scale = np.abs(g["FF_integrated"]).max()
    assert np.abs(o["FF_integrated"] - g["FF_integrated"]).max() < 1e-12 * scale
    assert np.abs(o["entry"] - g["entry"]).max() < 1e-12 * np.abs(g["entry"]).max()
    assert np.abs(o["exit"] - g["exit"]).max() < 1e-12 * np.abs(g["exit"]).max()
    if "cumulative" in g:
        assert o["cumulative"].shape == g["cumulative"].shape
        assert np.abs(o["cumulative"] - g["cumulative"]).max() < 1e-12 * np.abs(g["cumulative"]).max()


def test_trapz_weights():
    import oracle.hankel as oh
    from scipy import integrate

    x = np.sort(np.random.default_rng(0).uniform(0, 1, 17))
    y = np.random.default_rng(1).standard_normal(17)
    assert abs(np.sum(oh.trapz_weights(x) * y) - integrate.trapezoid(y, x=x)) < 1e-14


def test_radial_prefactor_matches_reference():
    """zr-modulated medium: the pre-factor table against the reference's own zr branch
    (Hankel_transform.py:302-399, fixture made by tests/golden/make_golden.py)."""
    from mma_gb300 import hankel as H

    g = np.load(os.path.join(GOLDEN, "prefactor_radial.npz"))
    H.XUV_index.set_constant_index(complex(g["n_xuv"][0], g["n_xuv"][1]))
    press = dict(zgrid=g["pressure_zgrid"], rgrid=g["pressure_rgrid"], value=g["pressure_value"])
    pre, renorm = H.pre_factor_table(g["zgrid"], g["ogrid"], "Ar", press, rgrid=g["rgrid"])
    assert renorm is None and bool(g["renorm_is_none"])
    assert pre.shape == g["pre"].shape
    assert np.abs(pre - g["pre"]).max() < 1e-12 * np.abs(g["pre"]).max()


def test_radial_profile_constant_in_r_is_the_plain_medium():
    """r branch: a radially constant profile gives the no-modulation pre-factor at every radius."""
    from mma_gb300 import hankel as H

    H.XUV_index.set_constant_index(complex(1 - 1e-5, 1e-7))
    z = np.linspace(-1e-3, 1e-3, 5)
    w = np.linspace(1e16, 3e16, 4)
    r = np.linspace(0.0, 1e-4, 6)
    pre_r, ren = H.pre_factor_table(z, w, "Ar", dict(rgrid=np.array([0.0, 2e-4]), value=np.array([0.8, 0.8])), rgrid=r)
    pre0, _ = H.pre_factor_table(z, w, "Ar", 0.8)
    assert ren is None
    for k in range(len(r)):
        assert np.allclose(pre_r[:, :, k], pre0, rtol=1e-14, atol=0)
