"""numpy restatement of the reference far-field integral (test infrastructure).

Follows Hankel/Hankel_transform.py:
  * FSources_provider (:29-80): planes zgrid[0:-1] (the last plane is dropped), source
    rows FSource[kz, omega, r];
  * get_propagation_pre_factor_function, no-modulation branch (:405-448):
        pre(z_k, w) = p exp(w (z_k disp(w) + (z_k - z_last) absorb(w))),
        renorm(k)   = exp((z_last - z_k) w absorb(w)),
    with disp = 1j (1/v_IR - 1/v_XUV) and absorb = (p/c) beta;
  * HankelTransform (:452-519):
        P[w, rho] = trapz_r( pre[r, w] e^{-i k r^2/(2 D)} r S[w, r] J0(k r rho / D) ),  k = w/c,
    the near-field factor optional;
  * Hankel_long (:523-686): D_k = distance - z_k per plane, z-trapezoid of the planes,
    cumulative results renormalised with renorm(k1) (k1, not k1+1: the reference's
    indexing is kept), entry and exit plane transforms.
Vectorised over (omega, rho, r) per plane; J0 from scipy.special.j0 (the same Cephes
routine behind the reference's scipy.special.jn(0, .)).
"""
import numpy as np
from scipy import special

C_LIGHT = 299792458.0  # shared_python/units.py:3


def trapz_weights(x):
    """Weights w with sum(w * y) == scipy.integrate.trapezoid(y, x) (Hankel_transform.py:22-27)."""
    x = np.asarray(x, dtype=np.float64)
    w = np.zeros_like(x)
    d = np.diff(x)
    w[:-1] += 0.5 * d
    w[1:] += 0.5 * d
    return w


def pre_factor_table(zgrid, ogrid, pressure=1.0, disp=None, absorb=None):
    """[Nz, No] complex pre-factors of the no-modulation branch and [Nz, No] renorm factors.

    disp, absorb: per-omega arrays (complex dispersion factor 1j*(1/v_IR - 1/v_XUV) and
    real absorption factor (p/c)*beta); None means the factor is switched off."""
    z = np.asarray(zgrid, dtype=np.float64)
    w = np.asarray(ogrid, dtype=np.float64)
    d = np.zeros_like(w, dtype=np.complex128) if disp is None else np.asarray(disp, dtype=np.complex128)
    a = np.zeros_like(w) if absorb is None else np.asarray(absorb, dtype=np.float64)
    pre = pressure * np.exp(w[None, :] * (z[:, None] * d[None, :] + (z[:, None] - z[-1]) * a[None, :]))
    renorm = np.exp((z[-1] - z[:, None]) * (w * a)[None, :])
    return pre, renorm


def constant_index_factors(ogrid, n_xuv, pressure=1.0, n_ir=1.0):
    """disp and absorb for a constant complex XUV index n = n0 + i beta (pressure-scaled
    deviation), as XUV_refractive_index.dispersion_function / beta_factor_ref return for a
    table with constant entries."""
    w = np.asarray(ogrid, dtype=np.float64)
    disp = 1j * pressure * (n_ir - n_xuv.real) / C_LIGHT * np.ones_like(w)
    absorb = (pressure / C_LIGHT) * n_xuv.imag * np.ones_like(w)
    return disp, absorb


def hankel_plane(ogrid, rgrid, S_plane, distance, rho, pre_row=None, near_field=True):
    """One HankelTransform: S_plane [No, Nr] -> [No, Nrho] complex128."""
    w = np.asarray(ogrid, dtype=np.float64)
    r = np.asarray(rgrid, dtype=np.float64)
    rho = np.asarray(rho, dtype=np.float64)
    k = w / C_LIGHT
    A = np.asarray(S_plane, dtype=np.complex128) * r[None, :]
    if near_field:
        A = A * np.exp(-1j * k[:, None] * r[None, :] ** 2 / (2.0 * distance))
    if pre_row is not None:  # [No], or [No, Nr] for a radially modulated medium (factor per radius, :505-512)
        pr = np.asarray(pre_row)
        A = A * (pr if pr.ndim == 2 else pr[:, None])
    A = A * trapz_weights(r)[None, :]
    out = np.empty((len(w), len(rho)), dtype=np.complex128)
    for i in range(len(w)):
        J = special.j0(k[i] * rho[:, None] * r[None, :] / distance)
        out[i] = J @ A[i]
    return out


def hankel_long(zgrid_full, rgrid, ogrid, S, distance, rho, pressure=1.0, disp=None, absorb=None, near_field=True,
                cumulative=False, pre=None):
    """Hankel_long on a static source S[kz, omega, r]; zgrid_full is the grid the source was
    given on (its last plane is dropped as FSources_provider does).

    Returns dict(FF_integrated [Nrho, No], entry, exit, planes [Nz, Nrho, No] and, when
    asked, cumulative [Nz-1, Nrho, No]).  ``pre`` overrides the no-modulation pre-factor."""
    z = np.asarray(zgrid_full, dtype=np.float64)[0:-1]
    if pre is None:
        pre, renorm = pre_factor_table(z, ogrid, pressure, disp, absorb)
    else:  # a given table: [Nz, No] or [Nz, No, Nr] (radially modulated medium, no renormalisation)
        renorm = np.ones((len(z), len(ogrid)))
    planes = np.stack([hankel_plane(ogrid, rgrid, S[k], distance - z[k], rho, pre[k], near_field).T
                       for k in range(len(z))])
    ff = np.zeros_like(planes[0])
    cum = []
    for k in range(len(z) - 1):
        ff = ff + 0.5 * (z[k + 1] - z[k]) * (planes[k] + planes[k + 1])
        if cumulative:
            cum.append(renorm[k][None, :] * ff)
    out = dict(FF_integrated=ff, entry=planes[0], exit=planes[-1], planes=planes)
    if cumulative:
        out["cumulative"] = np.stack(cum)
    return out
