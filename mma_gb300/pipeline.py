"""Microscopic-to-far-field on one GPU: the TDSE batch's source-term spectra stay in device
memory and feed the far-field integral directly.

The reference runs this as three programs joined by HDF5 files:

* the TDSE task farm (1DTDSE/sources/MPI-TDSE.c:163-329) computes one instance per macroscopic
  point n = kr + kz Nr and merge.py (1DTDSE/python/merge.py:98-106) writes
  FSourceTerm[kz, kr, omega] (a.u.);
* the far-field driver (Hankel/Hankel_long_medium_parallel_cluster.py:147-216) selects the
  harmonic window ko_min = FindInterval(ogrid/omega0, H_min), ko_max = FindInterval(ogrid/omega0,
  H_max), converts omega to SI (omega_au2SI, shared_python/mynumerics.py:324) and builds a
  FSources_provider on FSourceTerm[kz, 0:kr_max:kr_step, ko_min:ko_max:ko_step]^T with the last
  plane dropped (Hankel/Hankel_transform.py:29-80);
* Hankel_long (Hankel/Hankel_transform.py:523-686) integrates.

Here the three stages share HBM: ``microscopic_to_far_field`` propagates the batch
(``tdse_batch.run_batch``), views its spectra as [Nz, N_omega, Nr] without a copy, and passes them
to ``hankel.Hankel_long`` with the same selection arguments.
"""
import numpy as np
import torch

from . import hankel as H
from .tdse_batch import run_batch

# atomic unit of time, shared_python/units.py:3-4,19: TIMEau = elmass r_Bohr^2 / hbar
_HBAR = 1.0545718e-34
_ELMASS = 9.10938356e-31
_C = 299792458.0
_INV_ALPHA = 137.035999139
_R_BOHR = _HBAR * _INV_ALPHA / (_C * _ELMASS)
TIME_AU = _ELMASS * _R_BOHR ** 2 / _HBAR
OMEGA_AU2SI = 1.0 / TIME_AU


def find_interval(x, x0):
    """Index k with x[k] <= x0 < x[k+1]; x0 == x[-1] gives len(x) - 2; out of range raises
    LookupError (shared_python/mynumerics.py:35-60)."""
    x = np.asarray(x, dtype=np.float64)
    if x0 > x[-1] or x0 < x[0]:
        raise LookupError("out of range in FindInterval")
    k = int(np.searchsorted(x, x0, side="right")) - 1
    return min(k, len(x) - 2)


def harmonic_window(ogrid_au, omega0_au, harmonic_range, ko_step=1):
    """(ko_min, ko_max) of the far-field driver's selection ogrid[ko_min:ko_max:ko_step]
    (Hankel_long_medium_parallel_cluster.py:163-168)."""
    h = np.asarray(ogrid_au, dtype=np.float64) / float(omega0_au)
    return find_interval(h, harmonic_range[0]), find_interval(h, harmonic_range[-1])


def sources_from_spectra(Fsourceterm, n_r, n_z):
    """View a uniform batch's spectra [n_inst = n_z n_r, N_omega] (instance n = kr + kz n_r,
    MPI-TDSE.c:148,176-178) as the source [n_z, N_omega, n_r] the far-field provider slices."""
    F = Fsourceterm
    if F.dim() != 2 or F.shape[0] != n_r * n_z:
        raise ValueError("spectra must be [n_z * n_r, N_omega] with instance n = kr + kz * n_r")
    return F.view(n_z, n_r, F.shape[1]).permute(0, 2, 1)


def microscopic_to_far_field(grids, fields, dt_field, rgrid, zgrid, omega0_au, harmonic_range, rgrid_FF, distance,
                             precision="c64", ko_step=1, kr_step=1, kr_max="end", kz_step=1, grid_ids=None,
                             dt_req=None, tmax=None, **hankel_kwargs):
    """Propagate every macroscopic point and integrate the far field, all on the GPU.

    fields: float64 cuda tensor [Nz * Nr, n_f], instance n = kr + kz Nr (every instance with the
    same sampling, so one frequency grid).  rgrid, zgrid: macroscopic grids (SI).  omega0_au: the
    laser frequency (a.u.); harmonic_range = (H_min, H_max).  rgrid_FF, distance and
    ``hankel_kwargs`` are Hankel_long's.  Returns (TDSE BatchResult, Hankel_long result)."""
    n_r, n_z = len(rgrid), len(zgrid)
    if not (torch.is_tensor(fields) and fields.dim() == 2 and fields.shape[0] == n_r * n_z):
        raise ValueError("fields must be a [Nz * Nr, n_f] tensor")
    res = run_batch(grids, fields, dt_field, grid_ids=grid_ids, dt_req=dt_req, precision=precision, tmax=tmax)
    og_au = res["omegagrid"].cpu().numpy() if torch.is_tensor(res["omegagrid"]) else np.asarray(res["omegagrid"])
    ko_min, ko_max = harmonic_window(og_au, omega0_au, harmonic_range, ko_step)
    src = sources_from_spectra(res["Fsourceterm"], n_r, n_z)
    target = H.FSources_provider(np.asarray(zgrid), np.asarray(rgrid), OMEGA_AU2SI * og_au, FSource=src,
                                 ko_min=ko_min, ko_max=ko_max, ko_step=ko_step, kr_step=kr_step, kr_max=kr_max,
                                 kz_step=kz_step, device=fields.device)
    far = H.Hankel_long(target, distance, rgrid_FF, **hankel_kwargs)
    return res, far
