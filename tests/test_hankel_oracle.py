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
