"""The pipeline's HDF5 archives around the TDSE -> far-field path (through mma_gb300.h5io).

* ``read_cuprad_fields``: the driving fields and grids the MPI TDSE driver reads from the
  macroscopic archive (1DTDSE/sources/MPI-TDSE.c:96-190 with the paths of h5namelist.h:11-25):
  CUPRAD/outputs/output_field [z, t, r] in V/m, tgrid (s), rgrid, zgrid (m), coarsened by
  (kz_step, Nz_max), (kr_step, Nr_max) as coarsen_grid_real does (tools_algorithmic.c:54-65),
  converted to atomic units with the library's constants (constants.c:27-37).  Instances are
  numbered n = kr + kz Nr (MPI-TDSE.c:176-178), the order the batch API takes.
* ``write_ctdse_outputs``: a batch's results in the merged layout of 1DTDSE/python/merge.py:71-108
  under CTDSE/outputs/ -- per-point series [Nz, Nr, Nt] and spectra [Nz, Nr, Nomega(, 2)] in
  FP64 with their ``units`` attributes, the shared grids and ground-state data as the local
  files hold them (tools_hdf5.c prepare_local_output_fixed_print_grids_h5; MPI-TDSE.c:235-249).
* ``write_hankel_outputs``: a Hankel_long result under Hankel/outputs/ in the layout of
  Hankel/Hankel_long_medium_parallel_cluster.py:323-367 (complex arrays as a trailing re/im
  axis of 2, ``units`` attributes).
* ``read_fsource`` / ``FSources_provider(data_source="dynamic", h5_handle=..., h5_path=...)``:
  the far-field driver's source CTDSE/outputs/FSourceTerm [kz, kr, omega, re/im]
  (Hankel_transform.py:71-77).
"""
import math

import numpy as np
import torch

from . import h5io

# atomic units of time and electric field from the library's constants (constants.c:27-37)
_HBAR, _ELCHARGE, _ELMASS, _C = 1.054571800e-34, 1.602176565e-19, 9.10938356e-31, 299792458.0
_EPS0 = 1.0 / (4.0 * math.pi * 1e-7 * _C * _C)
_R_BOHR = 4.0 * math.pi * _EPS0 * _HBAR * _HBAR / (_ELMASS * _ELCHARGE * _ELCHARGE)
TIMEau = _ELMASS * _R_BOHR * _R_BOHR / _HBAR
EFIELDau = _HBAR * _HBAR / (_ELMASS * _R_BOHR ** 3 * _ELCHARGE)

CTDSE_OUTPUTS = "CTDSE/outputs"
HANKEL_OUTPUTS = "Hankel/outputs"
# merged per-point outputs and their units (merge.py:38-45); PopTot is not merged there
OUTPUT_UNITS = {"Efield": "[a.u.]", "FEfield": "[a.u.]", "SourceTerm": "[a.u.]", "FSourceTerm": "[a.u.]",
                "FEfieldM2": "[a.u.]", "FSourceTermM2": "[a.u.]", "PopInt": "[-]", "expval_x": "[a.u.]"}
FURTHER_UNITS = {"tgrid": "[a.u.]", "omegagrid": "[a.u.]", "Energy_of_the_ground_state": "[a.u.]",
                 "xgrid_micro": "[a.u.]", "ground_state": "[a.u.]", "zgrid_coarse": "[a.u.]",
                 "rgrid_coarse": "[a.u.]", "trg_a": "[a.u.]"}


def _open(f, mode="r"):
    return h5io.File(f, mode) if isinstance(f, str) else f


def coarsen(grid, k_step, n_max):
    """coarsen_grid_real (tools_algorithmic.c:54-65): the first n_max // k_step points taken
    k_step apart."""
    n = int(n_max) // int(k_step)
    grid = np.asarray(grid, dtype=np.float64)
    if n < 1 or (n - 1) * k_step >= grid.size:
        raise ValueError("coarsening (step %d, max %d) reaches beyond a grid of %d points" % (k_step, n_max, grid.size))
    return grid[0:n * k_step:k_step]


def read_cuprad_fields(archive, kz_step=None, kr_step=None, Nz_max=None, Nr_max=None):
    """Fields for the TDSE batch from a macroscopic archive.

    The coarsening parameters default to the archive's CTDSE/inputs/{kz_step, kr_step, Nz_max,
    Nr_max} (MPI-TDSE.c:110-120).  Returns dict(tgrid [Nt] a.u., fields [Nz_c Nr_c, Nt] a.u.
    float64, rgrid_coarse, zgrid_coarse (SI), n_r, n_z).  As the reference does, Nr_max beyond
    the archive's radial points is an error (MPI-TDSE.c:192-202)."""
    f = _open(archive)
    prm = {}
    for name, v in (("kz_step", kz_step), ("kr_step", kr_step), ("Nz_max", Nz_max), ("Nr_max", Nr_max)):
        prm[name] = int(v) if v is not None else int(np.asarray(f["CTDSE/inputs/" + name][()]).reshape(-1)[0])
    field = f["CUPRAD/outputs/output_field"]
    if field.ndim != 3:
        raise ValueError("output_field must be [z, t, r]")
    Nz, Nt, Nr = field.shape
    tgrid = np.asarray(f["CUPRAD/outputs/tgrid"][()], dtype=np.float64).reshape(-1)
    rgrid = np.asarray(f["CUPRAD/outputs/rgrid"][()], dtype=np.float64).reshape(-1)
    zgrid = np.asarray(f["CUPRAD/outputs/zgrid"][()], dtype=np.float64).reshape(-1)
    if tgrid.size != Nt or rgrid.size != Nr or zgrid.size != Nz:
        raise ValueError("grids do not match output_field [z, t, r] = %s" % (field.shape,))
    if prm["Nr_max"] > Nr:
        raise ValueError("'Nr_max' must be smaller than the number of radial points of the field")
    if prm["Nz_max"] > Nz:
        raise ValueError("'Nz_max' must be smaller than the number of longitudinal points of the field")
    rc = coarsen(rgrid, prm["kr_step"], prm["Nr_max"])
    zc = coarsen(zgrid, prm["kz_step"], prm["Nz_max"])
    E = np.asarray(field[()], dtype=np.float64)
    sel = E[0:zc.size * prm["kz_step"]:prm["kz_step"], :, 0:rc.size * prm["kr_step"]:prm["kr_step"]]
    fields = np.ascontiguousarray(sel.transpose(0, 2, 1).reshape(zc.size * rc.size, Nt)) / EFIELDau
    return dict(tgrid=tgrid / TIMEau, fields=fields, rgrid_coarse=rc, zgrid_coarse=zc, n_r=rc.size, n_z=zc.size)


def _np(a):
    return a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)


def write_ctdse_outputs(archive, res, n_r, n_z, rgrid_coarse, zgrid_coarse, grids=None, grid=0,
                        outputs=("Efield", "SourceTerm", "FSourceTerm", "FEfieldM2", "FSourceTermM2", "PopInt",
                                 "expval_x", "FEfield")):
    """Write a uniform batch's results (``run_batch``: instance n = kr + kz n_r) in the merged
    layout under CTDSE/outputs/.  ``grids`` (TDSEGrids) adds the microscopic grid, ground state,
    its energy and the soft-Coulomb parameter of grid ``grid``.  FEfield and FEfieldM2 are the
    DFT of each instance's output field with the source term's normalisation (calcFFTW3,
    tools_fftw3.c:84-143), by torch's FFT where the result tensors live.  ``archive`` is a path
    (appended to) or a writer from ``h5io.File(path, "w" | "a")``, which the caller closes."""
    f = _open(archive, "a")
    n = n_r * n_z
    series = {"Efield": "Efield", "SourceTerm": "sourceterm", "PopInt": "PopInt", "expval_x": "expval"}
    g = f.require_group(CTDSE_OUTPUTS)
    for key in outputs:
        if key in series:
            v = _np(res[series[key]])
            if v.shape[0] != n:
                raise ValueError("%s has %d instances, expected n_z * n_r = %d" % (key, v.shape[0], n))
            data = v.reshape(n_z, n_r, -1).astype(np.float64)
        elif key in ("FSourceTerm", "FSourceTermM2"):
            F = _np(res["Fsourceterm"]).reshape(n_z, n_r, -1)
            data = (np.stack([F.real, F.imag], axis=-1) if key == "FSourceTerm" else np.abs(F) ** 2)
        elif key in ("FEfield", "FEfieldM2"):
            F = _field_spectrum(res).reshape(n_z, n_r, -1)
            data = (np.stack([F.real, F.imag], axis=-1) if key == "FEfield" else np.abs(F) ** 2)
        else:
            raise ValueError("unknown output %r" % key)
        g.create_dataset(key, data=np.ascontiguousarray(data, dtype=np.float64)).attrs["units"] = \
            np.bytes_(OUTPUT_UNITS[key])
    tg = _np(res["tgrid"])
    further = {"tgrid": tg[0] if tg.ndim == 2 else tg, "omegagrid": _np(res["omegagrid"]),
               "rgrid_coarse": np.asarray(rgrid_coarse, np.float64), "zgrid_coarse": np.asarray(zgrid_coarse, np.float64)}
    if grids is not None:
        x = _np(grids.x(grid))
        psi0 = _np(grids.psi0(grid))
        further.update(xgrid_micro=x, ground_state=np.stack([psi0.real, psi0.imag], axis=1),
                       Energy_of_the_ground_state=np.array([float(grids.Einit[grid])]),
                       trg_a=np.array([float(grids.params[grid]["trg_a"])]))
    for k, v in further.items():
        g.create_dataset(k, data=np.asarray(v, dtype=np.float64)).attrs["units"] = np.bytes_(FURTHER_UNITS[k])
    if isinstance(archive, str):
        f.close()


def _field_spectrum(res):
    """dt/sqrt(2 pi) conj(DFT) of every instance's output field series (all Nt samples), as
    calcFFTW3 gives FEfield (tools_fftw3.c:84-143, called at singleTDSE.c:108), over the
    frequency grid of the source term."""
    E = res["Efield"]
    E = E if torch.is_tensor(E) else torch.from_numpy(np.asarray(E))
    tg = _np(res["tgrid"])
    t = tg[0] if tg.ndim == 2 else tg
    dt = float(t[1] - t[0])
    S = torch.fft.rfft(E.to(torch.float64), dim=-1)
    No = _np(res["omegagrid"]).size
    return (dt / math.sqrt(2.0 * math.pi)) * torch.conj(S[:, :No]).resolve_conj().cpu().numpy()


def write_hankel_outputs(archive, far):
    """A Hankel_long result under Hankel/outputs/ (Hankel_long_medium_parallel_cluster.py:
    323-367): FF_integrated, entry/exit plane transforms, ogrid and rgrid, and the cumulative
    fields and zgrid where the result has them."""
    f = _open(archive, "a")
    g = f.require_group(HANKEL_OUTPUTS)

    def cplx(name, a):
        a = np.asarray(a)
        g.create_dataset(name, data=np.stack([a.real, a.imag], axis=-1).astype(np.float64)).attrs["units"] = \
            np.bytes_("[arb. u.]")

    cplx("FF_integrated", far.FF_integrated)
    cplx("entry_plane_transform", far.entry_plane_transform)
    cplx("exit_plane_transform", far.exit_plane_transform)
    g.create_dataset("ogrid", data=np.asarray(far.ogrid, np.float64)).attrs["units"] = np.bytes_("[SI]")
    g.create_dataset("rgrid", data=np.asarray(far.rgrid, np.float64)).attrs["units"] = np.bytes_("[SI]")
    if hasattr(far, "cumulative_field"):
        cplx("cumulative_field", far.cumulative_field)
    if hasattr(far, "cumulative_field_no_norm"):
        cplx("cumulative_field_no_norm", far.cumulative_field_no_norm)
    if hasattr(far, "zgrid"):
        g.create_dataset("zgrid", data=np.asarray(far.zgrid, np.float64)).attrs["units"] = np.bytes_("[SI]")
    if isinstance(archive, str):
        f.close()


def read_fsource(dataset, n_planes, kz_step=1, kr_max=None, kr_step=1, ko_min=0, ko_max=None, ko_step=1):
    """The planes the far-field provider yields from CTDSE/outputs/FSourceTerm [kz, kr, omega,
    re/im] (Hankel_transform.py:71-77): plane k1 = FSourceTerm[k1 kz_step, kr, omega, 0] +
    i [..., 1], transposed to [omega, r].  Returns complex128 [n_planes, N_omega, N_r]."""
    a = np.asarray(dataset[()])
    if a.ndim != 4 or a.shape[-1] != 2:
        raise ValueError("FSourceTerm must be [kz, kr, omega, 2]")
    kr_max = a.shape[1] if kr_max is None else kr_max
    ko_max = a.shape[2] if ko_max is None else ko_max
    sel = a[0:n_planes * kz_step:kz_step, 0:kr_max:kr_step, ko_min:ko_max:ko_step]
    return np.ascontiguousarray((sel[..., 0] + 1j * sel[..., 1]).transpose(0, 2, 1))
