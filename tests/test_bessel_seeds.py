"""The far-field J0/J1 seeds (bessel01 in mma_gb300/csrc/hankel_common.cuh) restated in float32
arithmetic, on the CPU, against scipy: for x >= 3 the Abramowitz & Stegun 9.4.3/9.4.6 modulus and
phase with one reduced sin/cos (Cody-Waite reduction by pi/2, Taylor polynomials on |r| <= pi/4)
rotated by the small phase corrections.  Pins the accuracy the device function claims: the
approximations' own 1e-7 level (bound 2e-7), and 1e-7 for the reduced sin/cos."""
import numpy as np
import pytest

scipy_special = pytest.importorskip("scipy.special")
f = np.float32


def fma(a, b, c):  # float32 FMA: the float64 product of two float32 is exact
    return f(np.float64(a) * np.float64(b) + np.float64(c))


def poly(t, cs):
    acc = f(cs[0])
    for c in cs[1:]:
        acc = fma(t, acc, f(c))
    return acc


def reduce_2pi(yh, yl):
    kk = f(np.rint(f(yh * f(0.159154943))))
    r = fma(-kk, f(6.28125), yh)
    r = fma(-kk, f(1.93500518798828125e-3), r)
    r = fma(-kk, f(3.0199159819370158e-07), r)
    return f(r + yl)


def sincos_reduced(x):
    k = f(np.rint(f(x * f(0.636619772))))
    r = fma(-k, f(1.5703125), x)
    r = fma(-k, f(4.83826794896619e-4), r)
    r2 = f(r * r)
    s = f(r * poly(r2, [2.75573192e-6, -1.98412698e-4, 8.33333333e-3, -1.66666667e-1, 1.0]))
    c = poly(r2, [2.48015873e-5, -1.38888889e-3, 4.16666667e-2, -0.5, 1.0])
    q = int(k) & 3
    ss, cc = (c, s) if q & 1 else (s, c)
    return (-ss if q & 2 else ss), (-cc if (q + 1) & 2 else cc)


def sincos_small(p):
    p2 = f(p * p)
    return f(p * poly(p2, [8.33333333e-3, -1.66666667e-1, 1.0])), poly(p2, [4.16666667e-2, -0.5, 1.0])


F0 = [0.00014476, -0.00072805, 0.00137237, -0.00009512, -0.00552740, -0.00000077, 0.79788456]
P0 = [0.00013558, -0.00029333, -0.00054125, 0.00262573, -0.00003954, -0.04166397]
F1 = [-0.00020033, 0.00113653, -0.00249511, 0.00017105, 0.01659667, 0.00000156, 0.79788456]
P1 = [-0.00029166, 0.00079824, 0.00074348, -0.00637879, 0.00005650, 0.12499612]


def bessel01(y):
    yh = f(y)
    yl = f(y - np.float64(yh))
    t = f(f(3.0) / yh)
    red = reduce_2pi(yh, yl)
    sq = f(1.0 / np.sqrt(np.float64(yh)))
    sr, cr = sincos_reduced(red)
    a, b = f(cr + sr), f(cr - sr)
    f0, p0 = poly(t, F0), f(t * poly(t, P0))
    f1, p1 = poly(t, F1), f(t * poly(t, P1))
    s0, c0 = sincos_small(p0)
    s1, c1 = sincos_small(p1)
    J0 = f(f(f0 * sq) * f(f(0.707106781) * fma(c0, a, f(s0 * b))))
    J1 = f(f(f1 * sq) * f(f(0.707106781) * fma(s1, a, f(-c1 * b))))
    return J0, J1


def test_reduced_sincos():
    xs = np.linspace(-4.2, 3.6, 4001).astype(np.float32)
    err = max(max(abs(s - np.sin(np.float64(x))), abs(c - np.cos(np.float64(x))))
              for x in xs for s, c in [sincos_reduced(x)])
    assert err < 1e-7, err


def test_asymptotic_seeds_against_scipy():
    ys = np.concatenate([np.linspace(3.0, 40.0, 1500), np.random.default_rng(0).uniform(3.0, 3000.0, 2500)])
    e0 = e1 = 0.0
    for y in ys:
        J0, J1 = bessel01(y)
        e0 = max(e0, abs(J0 - scipy_special.j0(y)))
        e1 = max(e1, abs(J1 - scipy_special.j1(y)))
    assert e0 < 2e-7 and e1 < 2e-7, (e0, e1)  # measured 1.0e-7 and 1.25e-7


def test_small_angle_sincos():
    """sincos_small (and its packed form sincos_small_p, the same operations lane by lane): the
    Taylor polynomials to p^5 and p^4 on |p| <= 0.13, the range the far field's near-field phases
    and the seeds' phase corrections use; the remainders are below 6e-9, so float32 rounding sets
    the error."""
    ps = np.linspace(-0.13, 0.13, 4001).astype(np.float32)
    err = max(max(abs(s - np.sin(np.float64(p))), abs(c - np.cos(np.float64(p))))
              for p in ps for s, c in [sincos_small(p)])
    assert err < 1.2e-7, err
