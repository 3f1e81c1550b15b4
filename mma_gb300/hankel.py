"""The far-field integral on the GPU, mirroring Hankel/Hankel_transform.py.

Same names, arguments and results as the reference module:

* ``trapezoidal_integrator`` (:22) -- the only radial integrator; it is a marker
  here (the kernels apply trapezoid weights), other integrators raise.
* ``FSources_provider`` (:29-80) -- planes zgrid[0:-1:kz_step] (the last plane is
  dropped, as in the reference), source slices FSource[kz, omega, r]; the static
  source is moved to the GPU once.  'dynamic' sources are read from the HDF5 archive
  (CTDSE/outputs/FSourceTerm [kz, kr, omega, re/im]) by this package's own reader,
  mma_gb300.h5io, one plane at a time.
* ``get_propagation_pre_factor_function`` (:85-448) -- the no-modulation branch
  (scalar pressure) and the z-modulation branch (dict with 'zgrid', 'value'),
  returning (pre_factor(kz) -> [Nr, No], exp_renorm(kz) -> [No]) like the reference.
* ``HankelTransform`` (:452-519) -> [No, Nrho] complex128.
* ``Hankel_long`` (:523-686) -- FF_integrated [Nrho, No], entry/exit planes,
  cumulative results.  ``form="plain"`` runs the reference's arithmetic in FP64
  (CUDA kernels in mma_gb300/csrc/hankel.cu); ``form="fast"`` runs the chosen
  form (Bessel multiplication theorem, z-first contraction, FP32 with float-float
  phases) and records its truncation bound in ``self.fast_plan``.

Refractive index: the reference reads f1/f2 tables through XUV_refractive_index
(HDF5).  Here ``XUV_index`` is a provider with the same two functions; by default it
models a constant complex XUV index (``XUV_index.set_constant_index``);
``XUV_index.load_tables(directory)`` reads the CXRO/NIST text tables those HDF5 tables are
made from.
"""
import ctypes
import os
from ctypes import POINTER, Structure, c_double, c_int, c_int64, c_size_t, c_void_p

import numpy as np
import torch

from ._lib import load

C_LIGHT = 299792458.0  # shared_python/units.py:3


# ------------------------------------------------------------------------------ C-ABI records
class HankelProblem(Structure):
    _fields_ = [("n_omega", c_int64), ("n_r", c_int64), ("n_z", c_int64), ("n_rho", c_int64), ("distance", c_double),
                ("near_field", c_int64), ("source_c128", c_int64), ("plane_stride", c_int64),
                ("omega_stride", c_int64), ("pre_radial", c_int64)]


class FastPlan(Structure):
    _fields_ = [("d_ref", c_double), ("sigma", c_double), ("n_terms", c_int64), ("y_max", c_double),
                ("trunc_bound", c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HankelError(RuntimeError):
    pass


def _sig():
    lib = load()
    if getattr(lib, "_mma_hankel_sig", False):
        return lib
    P = POINTER(HankelProblem)
    lib.mma_hankel_plain.argtypes = [P, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_int, c_void_p, c_void_p]
    lib.mma_hankel_plain.restype = c_int
    lib.mma_hankel_fast_plan.argtypes = [POINTER(c_double), c_int64, c_double, c_double, c_double, c_double,
                                         c_double, POINTER(FastPlan)]
    lib.mma_hankel_fast_plan.restype = c_int
    lib.mma_hankel_fast_scratch_bytes.argtypes = [P, POINTER(FastPlan)]
    lib.mma_hankel_fast_scratch_bytes.restype = c_size_t
    lib.mma_hankel_fast.argtypes = [P, POINTER(FastPlan), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_void_p]
    lib.mma_hankel_fast.restype = c_int
    lib.mma_hankel_planes_tc_scratch_bytes.argtypes = [P, POINTER(FastPlan)]
    lib.mma_hankel_planes_tc_scratch_bytes.restype = c_size_t
    lib.mma_hankel_planes_tc.argtypes = [P, POINTER(FastPlan), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_size_t, c_void_p]
    lib.mma_hankel_planes_tc.restype = c_int
    lib.mma_hankel_planes_tc_prepare.argtypes = [P, POINTER(FastPlan), c_void_p, c_void_p, c_void_p, c_void_p,
                                                 c_void_p, c_void_p, c_size_t, c_void_p]
    lib.mma_hankel_planes_tc_prepare.restype = c_int
    lib.mma_hankel_planes_tc_run.argtypes = [P, POINTER(FastPlan), c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                             c_void_p, c_void_p, c_size_t, c_void_p]
    lib.mma_hankel_planes_tc_run.restype = c_int
    lib.mma_hankel_planes_tc_status.argtypes = [P, POINTER(FastPlan), c_void_p, c_void_p]
    lib.mma_hankel_planes_tc_status.restype = c_int
    lib.mma_hankel_set_stage1.argtypes = [c_int]
    lib.mma_hankel_set_stage1.restype = c_int
    lib.mma_hankel_copy_block.argtypes = [c_void_p, c_void_p, c_int64, c_int64, c_int64, c_void_p]
    lib.mma_hankel_copy_block.restype = c_int
    lib.mma_hankel_ff_from_planes.argtypes = [P, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
    lib.mma_hankel_ff_from_planes.restype = c_int
    lib.mma_hankel_fast_status.argtypes = [P, POINTER(FastPlan), c_void_p, c_void_p]
    lib.mma_hankel_fast_status.restype = c_int
    lib._mma_hankel_sig = True
    return lib


def _check(rc, what):
    if rc != 0:
        raise HankelError("%s failed with status %d" % (what, rc))


# ------------------------------------------------------------------------------ refractive index
# physical constants of shared_python/units.py:3-7,16-19 (the reference's values)
_HBAR, _INV_ALPHA, _ELCHARGE, _ELMASS = 1.0545718e-34, 137.035999139, 1.602176565e-19, 9.10938356e-31
_ALPHA = 1.0 / _INV_ALPHA
_R_BOHR = _HBAR * _INV_ALPHA / (C_LIGHT * _ELMASS)
_R_ELECTRON = _R_BOHR * _ALPHA ** 2
_TIME_AU = _ELMASS * _R_BOHR ** 2 / _HBAR
N_REF_DEFAULT = 2.7e25  # XUV_refractive_index.py:122

# tabulated scattering factors: gas -> files, in the directory layout of shared_python/XUV_tables
TABLE_FILES = {
    "He_Henke": ("he.nff",), "Ne_Henke": ("ne.nff",), "Ar_Henke": ("ar.nff",), "Kr_Henke": ("kr.nff",),
    "Xe_Henke": ("xe.nff",),
    "He_NIST": ("he_f1_NIST.txt", "he_f2_NIST.txt"), "Ne_NIST": ("ne_f1_NIST.txt", "ne_f2_NIST.txt"),
    "Ar_NIST": ("ar_f1_NIST.txt", "ar_f2_NIST.txt"), "Kr_NIST": ("kr_f1_NIST.txt", "kr_f2_NIST.txt"),
    "Xe_NIST": ("xe_f1_NIST.txt", "xe_f2_NIST.txt"),
}


def _omega_si_to_ev(omega):
    """mynumerics.ConvertPhoton(omega, 'omegaSI', 'eV') (mynumerics.py:313,325)."""
    return np.asarray(omega, dtype=float) * _TIME_AU / (_ELCHARGE / (_ELMASS * _ALPHA ** 2 * C_LIGHT ** 2))


def _omega_si_to_lambda(omega):
    """mynumerics.ConvertPhoton(omega, 'omegaSI', 'lambdaSI') (mynumerics.py:313,322)."""
    w_au = np.asarray(omega, dtype=float) * _TIME_AU
    return 2.0 * np.pi * _HBAR / (w_au * _ELMASS * C_LIGHT * _ALPHA ** 2)


def _read_columns(path, skip, cols):
    """Rows of whitespace-separated numbers after `skip` header lines, blank lines ignored (the
    parsing of shared_python/make_table.py)."""
    out = []
    with open(path) as f:
        for k, line in enumerate(f):
            parts = line.split()
            if k < skip or not parts:
                continue
            out.append([float(parts[c]) for c in cols])
    return np.asarray(out, dtype=float)


class _XUVIndex:
    """XUV refractive index provider with the interface of the reference's XUV_refractive_index
    (gases, dispersion_function :125-161, beta_factor_ref :164-194).

    Two sources:
    * ``set_constant_index(n)``: a constant complex index n = n0 + i beta per reference density
      (the dispersion term scales with pressure like the tabulated one) -- the default;
    * ``load_tables(directory)``: the tabulated scattering factors f1, f2 of the CXRO (Henke,
      ``*.nff``: E [eV], f1, f2 after one header line) and NIST (``*_f1_NIST.txt``,
      ``*_f2_NIST.txt``: E [keV], f after three header lines) tables in the directory layout of
      shared_python/XUV_tables, linearly interpolated in photon energy (ValueError outside the
      table), with n_XUV = 1 - p N_ref r_e lambda^2 f1/(2 pi) and beta = N_ref r_e lambda^2 f2/(2 pi).
    """

    def __init__(self):
        self.set_constant_index(complex(1 - 1e-5, 1e-7))

    def set_constant_index(self, n, gases=("Ar_Henke", "Ar_NIST", "Ne_Henke", "He_Henke", "Kr_Henke", "Xe_Henke")):
        self.mode = "constant"
        self.n = complex(n)
        self.gases = list(gases)
        self.tables = {}

    def load_tables(self, directory, gases=None):
        tables = {}
        for gas, files in TABLE_FILES.items():
            if gases is not None and gas not in gases:
                continue
            paths = [os.path.join(directory, f) for f in files]
            if not all(os.path.exists(p) for p in paths):
                continue
            if len(files) == 1:
                t = _read_columns(paths[0], 1, (0, 1, 2))
                tables[gas] = (t[:, 0], t[:, 1], t[:, 0], t[:, 2])
            else:
                t1 = _read_columns(paths[0], 3, (0, 1))
                t2 = _read_columns(paths[1], 3, (0, 1))
                tables[gas] = (1e3 * t1[:, 0], t1[:, 1], 1e3 * t2[:, 0], t2[:, 1])
        if not tables:
            raise FileNotFoundError("no scattering-factor tables found in %s" % directory)
        self.mode = "tables"
        self.tables = tables
        self.gases = sorted(tables)

    @staticmethod
    def _interp(E, x, y):
        E = np.asarray(E, dtype=float)
        if np.any(E < x[0]) or np.any(E > x[-1]):
            raise ValueError("photon energy outside the scattering-factor table")
        return np.interp(E, x, y)

    def getf1(self, gas, E):
        x1, f1, _, _ = self.tables[gas]
        return self._interp(E, x1, f1)

    def getf2(self, gas, E):
        _, _, x2, f2 = self.tables[gas]
        return self._interp(E, x2, f2)

    def dispersion_function(self, omega, pressure, gas, n_IR=1.0, N_ref=N_REF_DEFAULT):
        if self.mode == "constant":
            return pressure * (n_IR - self.n.real) / C_LIGHT * np.ones_like(np.asarray(omega, dtype=float))
        f1 = self.getf1(gas, _omega_si_to_ev(omega))
        if np.any(f1 < -9998.0):
            raise ValueError("f1-scattering coefficient not listed for this frequency.")
        lam = _omega_si_to_lambda(omega)
        n_xuv = 1.0 - pressure * N_ref * _R_ELECTRON * (lam ** 2 * f1 / (2.0 * np.pi))
        return 1.0 / (C_LIGHT / n_IR) - 1.0 / (C_LIGHT / n_xuv)

    def beta_factor_ref(self, omega, gas, N_ref=N_REF_DEFAULT):
        if self.mode == "constant":
            return self.n.imag * np.ones_like(np.asarray(omega, dtype=float))
        f2 = self.getf2(gas, _omega_si_to_ev(omega))
        lam = _omega_si_to_lambda(omega)
        return N_ref * _R_ELECTRON * (lam ** 2 * f2 / (2.0 * np.pi))


XUV_index = _XUVIndex()


def trapezoidal_integrator(y, x):
    """Marker for the reference's default radial integrator (scipy trapezoid, :22-27)."""
    from scipy import integrate

    return integrate.trapezoid(y, x=x)


# ------------------------------------------------------------------------------ sources
class FSources_provider:
    """Planes and source of a long medium (Hankel_transform.py:29-80)."""

    def __init__(self, zgrid, rgrid, ogrid, data_source="static", FSource=None, h5_handle=None, h5_path=None,
                 ko_min=0, ko_step=1, ko_max="end", kr_step=1, kr_max="end", kz_step=1, device="cuda"):
        if ko_max == "end":
            ko_max = len(ogrid)
        if kr_max == "end":
            kr_max = len(rgrid)
        self.zgrid = np.asarray(zgrid)[0:-1:kz_step]
        self.rgrid = np.asarray(rgrid)[0:kr_max:kr_step]
        self.ogrid = np.asarray(ogrid)[ko_min:ko_max:ko_step]
        if data_source == "static":
            nz = len(self.zgrid)
            if torch.is_tensor(FSource):
                S = FSource[0:nz * kz_step:kz_step, ko_min:ko_max:ko_step, 0:kr_max:kr_step]
            else:
                S = torch.from_numpy(np.ascontiguousarray(
                    np.asarray(FSource)[0:nz * kz_step:kz_step, ko_min:ko_max:ko_step, 0:kr_max:kr_step]))
            if S.dtype not in (torch.complex64, torch.complex128):
                S = S.to(torch.complex128)
            self.source = S.to(device).contiguous()
        elif data_source == "dynamic":
            # h5_handle[h5_path] = FSourceTerm [kz, kr, omega, re/im] (Hankel_transform.py:71-77),
            # read once through mma_gb300.h5io (or any handle whose dataset gives numpy arrays)
            from .archive import read_fsource

            S = read_fsource(h5_handle[h5_path], len(self.zgrid), kz_step=kz_step, kr_max=kr_max, kr_step=kr_step,
                             ko_min=ko_min, ko_max=ko_max, ko_step=ko_step)
            self.source = torch.from_numpy(S).to(device).contiguous()
        else:
            raise ValueError("Wrongly specified input of the class.")

        def _planes():
            for k in range(self.source.shape[0]):
                yield self.source[k]

        self.Fsource_plane = _planes()


# ------------------------------------------------------------------------------ pre-factor
def get_propagation_pre_factor_function(zgrid, rgrid, ogrid, preset_gas="vacuum", pressure=1.0,
                                        absorption_tables="Henke", include_absorption=True, dispersion_tables="Henke",
                                        include_dispersion=True, effective_IR_refrective_index=1.0):
    """(pre_factor, exp_renorm) as in Hankel_transform.py:85-448 (no-modulation :405-448,
    z-modulation :146-239, radially modulated :242-399).  Returns numpy closures; pre_factor(kz)
    is [Nr, No] (the orientation HankelTransform reads, :505-512); ``pre_table`` gives [Nz, No]
    or [Nz, No, Nr].  A radially modulated medium has no renormalisation (None), as in the
    reference."""
    pre_tab, renorm_tab = pre_factor_table(zgrid, ogrid, preset_gas, pressure, absorption_tables, include_absorption,
                                           dispersion_tables, include_dispersion, effective_IR_refrective_index,
                                           rgrid=rgrid)
    Nr = len(rgrid)

    def pre_factor(kz):
        if pre_tab.ndim == 3:
            return pre_tab[kz].T
        return np.outer(np.ones(Nr), pre_tab[kz])

    pre_factor.pre_table = pre_tab
    if renorm_tab is None:
        return pre_factor, None

    def exp_renorm(kz):
        return renorm_tab[kz]

    pre_factor.pre_table = pre_tab
    exp_renorm.table = renorm_tab
    return pre_factor, exp_renorm


def _radial_pre_factor(z, r, w, gas, pressure, absorption_tables, include_absorption, dispersion_tables,
                       include_dispersion, n_ir):
    """[Nz, No, Nr] pre-factor of a radially modulated medium (Hankel_transform.py:242-399).

    * zr branch (pressure with 'zgrid', 'rgrid', 'value'[Nz_table, Nr_table], :302-399): the
      pressure rows interpolated in r onto the computational radii (edge values outside), then per
      radius the pressure interpolated onto the planes and, per frequency, the cumulative
      trapezoid along the table's z of the dispersion function and of the pressure (absorption,
      with beta of the *dispersion* tables as in :366-370), interpolated onto the planes:
          pre[z, w, r] = p(z, r) exp(w (i int disp dz + (1/c) beta int p dz)).
    * r branch (pressure with 'rgrid', 'value'[Nr_table], :242-299): a radial profile constant
      along z.  The reference's branch does not run (it indexes with k1 before defining it, :250,
      and uses an undefined dispersion_factor, :295); this implements its evident intent, the
      no-modulation formula (:405-448) with the local pressure p(r).
    The reference returns the zr table per plane as [omega, r] while HankelTransform reads it as
    [r, omega] (:505-512); here the factor of (plane, frequency, radius) multiplies that radius's
    integrand, which is what both functions describe."""
    from scipy import integrate, interpolate

    pr_r = np.asarray(pressure["rgrid"], dtype=np.float64)
    val = np.asarray(pressure["value"], dtype=np.float64)
    Nz, No, Nr = len(z), len(w), len(r)
    pre = np.empty((Nz, No, Nr), dtype=np.complex128)

    def on_r(row):  # :247-254, :316-323
        return interpolate.interp1d(pr_r, row, bounds_error=False, fill_value=(row[0], row[-1]), copy=False)(r)

    if "zgrid" not in pressure:
        p_r = on_r(val if val.ndim == 1 else val[0])
        beta = XUV_index.beta_factor_ref(w, gas + "_" + absorption_tables) if include_absorption else None
        for kr in range(Nr):
            if include_dispersion:
                disp = 1j * XUV_index.dispersion_function(w, p_r[kr], gas + "_" + dispersion_tables, n_IR=n_ir)
            else:
                disp = 1j * (n_ir - 1.0) / C_LIGHT * np.ones_like(w)
            absorb = (p_r[kr] / C_LIGHT) * beta if include_absorption else np.zeros_like(w)
            pre[:, :, kr] = p_r[kr] * np.exp(w[None, :] * (z[:, None] * disp[None, :] +
                                                          (z[:, None] - z[-1]) * absorb[None, :]))
        return pre
    pz = np.asarray(pressure["zgrid"], dtype=np.float64)
    p_rg = np.stack([on_r(val[k]) for k in range(len(pz))])  # [Nz_table, Nr]
    beta_d = XUV_index.beta_factor_ref(w, gas + "_" + dispersion_tables) if include_absorption else None
    for kr in range(Nr):
        col = p_rg[:, kr]
        p_loc = interpolate.interp1d(pz, col, bounds_error=False, fill_value=(col[0], col[-1]), copy=False)(z)
        if include_dispersion:
            dfun = XUV_index.dispersion_function(w[:, None], col[None, :], gas + "_" + dispersion_tables, n_IR=n_ir)
            integ = integrate.cumulative_trapezoid(np.broadcast_to(dfun, (No, len(pz))), x=pz, initial=0.0, axis=1)
            disp = 1j * interpolate.interp1d(pz, integ, axis=1, bounds_error=False,
                                             fill_value=(integ[:, 0], integ[:, -1]), copy=False)(z)
        else:
            disp = 1j * (n_ir - 1.0) / C_LIGHT * np.ones((No, Nz))
        if include_absorption:
            ib = beta_d[:, None] * integrate.cumulative_trapezoid(col, x=pz, initial=0.0)[None, :]
            absf = (1.0 / C_LIGHT) * interpolate.interp1d(pz, ib, axis=1, bounds_error=False,
                                                          fill_value=(ib[:, 0], ib[:, -1]), copy=False)(z)
        else:
            absf = 0.0
        pre[:, :, kr] = (p_loc[None, :] * np.exp(w[:, None] * (disp + absf))).T
    return pre


def pre_factor_table(zgrid, ogrid, preset_gas="vacuum", pressure=1.0, absorption_tables="Henke",
                     include_absorption=True, dispersion_tables="Henke", include_dispersion=True,
                     effective_IR_refrective_index=1.0, rgrid=None):
    """Pre-factor and renormalisation tables (the reference's closures evaluated): [Nz, No], or
    [Nz, No, Nr] for a radially modulated medium (pressure with 'rgrid'; needs `rgrid`; no
    renormalisation, as in the reference)."""
    z = np.asarray(zgrid, dtype=np.float64)
    w = np.asarray(ogrid, dtype=np.float64)
    n_ir = effective_IR_refrective_index
    if isinstance(pressure, dict):
        if "rgrid" in pressure:
            if rgrid is None:
                raise ValueError("a radially modulated medium needs the radial grid")
            return _radial_pre_factor(z, np.asarray(rgrid, dtype=np.float64), w, preset_gas, pressure,
                                      absorption_tables, include_absorption, dispersion_tables, include_dispersion,
                                      n_ir), None
        from scipy import integrate, interpolate

        pz, pv = np.asarray(pressure["zgrid"]), np.asarray(pressure["value"])
        p_loc = interpolate.interp1d(pz, pv, bounds_error=False, fill_value=(pv[0], pv[-1]), copy=False)(z)
        pre = np.empty((len(z), len(w)), dtype=np.complex128)
        absw = np.empty((len(z), len(w)))
        for k1 in range(len(w)):
            if include_dispersion:
                integrand = XUV_index.dispersion_function(w[k1], pv, preset_gas + "_" + dispersion_tables, n_IR=n_ir)
                ph = integrate.cumulative_trapezoid(integrand, x=pz, initial=0.0)
                disp = 1j * interpolate.interp1d(pz, ph, bounds_error=False, fill_value=(ph[0], ph[-1]), copy=False)(z)
            else:
                disp = 1j * (n_ir - 1.0) / C_LIGHT
            if include_absorption:
                ib = XUV_index.beta_factor_ref(w[k1], preset_gas + "_" + absorption_tables) * \
                    integrate.cumulative_trapezoid(pv, x=pz, initial=0.0)
                absf = (1.0 / C_LIGHT) * interpolate.interp1d(pz, ib, bounds_error=False, fill_value=(ib[0], ib[-1]),
                                                              copy=False)(z)
                absw[:, k1] = w[k1] * absf
                absf = absf - absf[-1]
            else:
                absf = 0.0
                absw[:, k1] = 0.0
            pre[:, k1] = p_loc * np.exp(w[k1] * (disp + absf))
        renorm = np.exp(absw[-1][None, :] - absw)
        return pre, renorm
    if include_dispersion:
        disp = 1j * XUV_index.dispersion_function(w, pressure, preset_gas + "_" + dispersion_tables, n_IR=n_ir)
    else:
        disp = 1j * (n_ir - 1.0) / C_LIGHT * np.ones_like(w)
    if include_absorption:
        absorb = (pressure / C_LIGHT) * XUV_index.beta_factor_ref(w, preset_gas + "_" + absorption_tables)
    else:
        absorb = np.zeros_like(w)
    pre = pressure * np.exp(w[None, :] * (z[:, None] * disp[None, :] + (z[:, None] - z[-1]) * absorb[None, :]))
    renorm = np.exp((z[-1] - z[:, None]) * (w * absorb)[None, :])
    return pre, renorm


# ------------------------------------------------------------------------------ kernels
def _dev(a, device, dtype=torch.float64):
    """A grid or table on the device.  Host data goes through pinned memory as an asynchronous copy
    on the current stream, so the host does not wait for the stream's earlier work."""
    if torch.is_tensor(a):
        if a.is_cuda:  # already on the device: no copy
            return a.to(device=device, dtype=dtype).contiguous()
        return a.to(dtype).contiguous().pin_memory().to(device, non_blocking=True)
    a = np.ascontiguousarray(a, dtype=np.dtype(str(dtype).replace("torch.", "")))
    if not a.flags.writeable:  # e.g. a view of a read-only archive buffer: torch wants writable memory
        a = a.copy()
    return torch.from_numpy(a).pin_memory().to(device, non_blocking=True)


TC_MIN_PLANES = 16  # from this many requested planes the fast form computes them on the tensor cores
SERIES_PLANES = 2  # up to this many planes the fast pass evaluates inside its series stage


def set_stage1_form(form):
    """Stage 1 of the fast form (the z contraction): "cuda" (default) runs it on the CUDA cores
    (FP32 FMAs); "tc" runs it on the tensor cores where it applies (16 series terms, complex64
    source rows on 16-byte boundaries, pre-factors per (plane, frequency)) as a TF32
    split-precision GEMM, which on config 3 is slower and about 20 times less accurate.  Other
    problems always take the CUDA cores."""
    if form not in ("tc", "cuda"):
        raise ValueError("stage-1 form must be 'tc' or 'cuda'")
    _check(_sig().mma_hankel_set_stage1(0 if form == "tc" else 1), "mma_hankel_set_stage1")


STREAM_BLOCK = 256  # frequencies per block when a pinned host source is uploaded while computing


def far_field(ogrid, rgrid, zgrid, rho, source, distance, pre_table=None, near_field=True, planes=(), form="plain",
              tol=1e-9, stream=None, planes_via="auto", ff_via="auto", _events=None, _omega_max=None, _grids=None):
    """Run the far-field kernels.  source: torch complex tensor [Nz, No, Nr] with r contiguous (on
    the GPU, or on the host: a host tensor is copied there first; a pinned host tensor, for the
    fast form with at most two planes, is uploaded in blocks of STREAM_BLOCK frequencies on a
    second stream while the blocks already on the device are computed -- the same result as the
    one-shot call, since every frequency is independent and all blocks share one plan).
    Returns (FF [Nrho, No] complex128 tensor, {plane: [Nrho, No] tensor}, fast plan dict or None).

    With form="fast", requested planes are computed in the fast pass (planes_via="direct": up to
    two planes, such as the entry and exit planes, by the same multiplication-theorem series inside
    its second stage, sharing its Bessel evaluations; more by one FP32 J0 per term) or by the
    tensor-core split-precision GEMM (planes_via="tc"); "auto" takes the tensor cores from
    TC_MIN_PLANES planes on, where the problem fits them.
    FF_integrated comes from the fast form's z-first series (ff_via="fast"), or, when every plane
    is computed on the tensor cores, as the z trapezoid of those planes (ff_via="planes": the
    quantity the cumulative results end on, at the planes' accuracy, without the series pass);
    "auto" takes "planes" in that case and "fast" otherwise."""
    lib = _sig()
    if not source.is_cuda:  # the kernels take device pointers only: a host source is copied first
        if (form == "fast" and source.is_pinned() and source.is_contiguous() and source.dim() == 3
                and source.shape[1] > STREAM_BLOCK and len(set(planes)) <= SERIES_PLANES):
            return _far_field_streamed(ogrid, rgrid, zgrid, rho, source, distance, pre_table, near_field, planes,
                                       tol, stream, planes_via, ff_via)
        source = source.to(torch.device("cuda", torch.cuda.current_device()))
    dev = source.device
    Nz, No, Nr = source.shape
    if len(zgrid) != Nz or len(ogrid) != No or len(rgrid) != Nr:
        raise ValueError("source shape does not match the grids")
    # planes and frequencies may be strided (a frequency block of a larger source); r is contiguous
    S = source if source.stride(2) == 1 and source.stride(1) >= Nr and source.stride(0) >= 0 else source.contiguous()
    radial = pre_table is not None and np.ndim(pre_table) == 3
    if pre_table is not None and tuple(np.shape(pre_table)) not in ((Nz, No), (Nz, No, Nr)):
        raise ValueError("pre-factor must be [Nz, No] or [Nz, No, Nr]")
    prob = HankelProblem(No, Nr, Nz, len(rho), float(distance), int(bool(near_field)),
                         int(S.dtype == torch.complex128), S.stride(0), S.stride(1), int(radial))
    strm = stream or torch.cuda.current_stream(dev)
    with torch.cuda.stream(strm):  # uploads and allocations on the call's stream
        return _far_field_on(lib, strm, prob, S, ogrid, rgrid, zgrid, rho, distance, pre_table, planes, form, tol,
                             planes_via, ff_via, _events, _omega_max, _grids)


def _far_field_on(lib, strm, prob, S, ogrid, rgrid, zgrid, rho, distance, pre_table, planes, form, tol, planes_via,
                  ff_via, _events, _omega_max, _grids):
    dev = S.device
    Nz, No, Nr = S.shape
    # _grids: the grids already on the device (the host arrays still give the plan)
    og, rg, zg, rh = _grids if _grids is not None else (_dev(a, dev) for a in (ogrid, rgrid, zgrid, rho))
    pre = None
    if pre_table is not None:  # a device tensor is used in place; a host table is copied once per call
        pre = _dev(pre_table, dev, torch.complex128)
    ff = torch.zeros(len(rho), No, dtype=torch.complex128, device=dev)
    planes = sorted(set(int(p) % Nz for p in planes))
    slot = None
    pl = None
    if planes:
        if len(planes) <= 8:  # built on the device: no copy to queue behind other transfers
            slot = torch.full((Nz,), -1, dtype=torch.int64, device=dev)
            for i, p in enumerate(planes):
                slot[p:p + 1].fill_(i)  # a fill kernel (no host copy, so a graph capture takes it)
        else:
            s = np.full(Nz, -1, dtype=np.int64)
            for i, p in enumerate(planes):
                s[p] = i
            slot = _dev(s, dev, torch.int64)
        # every element of a requested plane is written by each form's kernels
        pl = torch.empty(len(planes), len(rho), No, dtype=torch.complex128, device=dev)
    st = ctypes.c_void_p(strm.cuda_stream)
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    plan_d = None
    if form == "plain":
        _check(lib.mma_hankel_plain(ctypes.byref(prob), og.data_ptr(), rg.data_ptr(), zg.data_ptr(), rh.data_ptr(),
                                    S.data_ptr(), ptr(pre), ff.data_ptr(), ptr(slot), len(planes), ptr(pl), st),
               "mma_hankel_plain")
    elif form == "fast":
        zh = np.ascontiguousarray(_np(zgrid), dtype=np.float64)
        plan = FastPlan()
        om = float(np.max(np.abs(_np(ogrid)))) if _omega_max is None else float(_omega_max)
        _check(lib.mma_hankel_fast_plan(zh.ctypes.data_as(POINTER(c_double)), Nz, float(distance),
                                        om, float(np.max(np.abs(_np(rgrid)))),
                                        float(np.max(np.abs(_np(rho)))), float(tol), ctypes.byref(plan)),
               "mma_hankel_fast_plan")
        nb = lib.mma_hankel_fast_scratch_bytes(ctypes.byref(prob), ctypes.byref(plan))
        scratch = torch.empty(int(nb), dtype=torch.uint8, device=dev)
        ntc = int(lib.mma_hankel_planes_tc_scratch_bytes(ctypes.byref(prob), ctypes.byref(plan))) if planes else 0
        if planes_via not in ("auto", "tc", "direct"):
            raise ValueError("planes_via must be 'auto', 'tc' or 'direct'")
        use_tc = bool(planes) and ntc > 0 and (planes_via == "tc" or (planes_via == "auto" and
                                                                      len(planes) >= TC_MIN_PLANES))
        if planes_via == "tc" and planes and ntc == 0:
            raise HankelError("the tensor-core plane form does not support this problem (n_r > 1024 or > 32 terms)")
        if ff_via not in ("auto", "fast", "planes"):
            raise ValueError("ff_via must be 'auto', 'fast' or 'planes'")
        ff_planes = use_tc and len(planes) == Nz and ff_via in ("auto", "planes")
        if ff_via == "planes" and not ff_planes:
            raise HankelError("ff_via='planes' needs every plane computed on the tensor cores")
        if not ff_planes:
            _check(lib.mma_hankel_fast(ctypes.byref(prob), ctypes.byref(plan), og.data_ptr(), rg.data_ptr(),
                                       zg.data_ptr(), rh.data_ptr(), S.data_ptr(), ptr(pre), ff.data_ptr(),
                                       None if use_tc else ptr(slot), 0 if use_tc else len(planes),
                                       None if use_tc else ptr(pl), scratch.data_ptr(), int(nb), st), "mma_hankel_fast")
        if use_tc:
            tcs = torch.empty(ntc, dtype=torch.uint8, device=dev)
            _check(lib.mma_hankel_planes_tc_prepare(ctypes.byref(prob), ctypes.byref(plan), og.data_ptr(),
                                                    rg.data_ptr(), zg.data_ptr(), S.data_ptr(), ptr(pre),
                                                    tcs.data_ptr(), ntc, st), "mma_hankel_planes_tc_prepare")
            if _events is not None:  # (start, end) CUDA events around the tensor-core kernel
                _events[0].record(strm)
            _check(lib.mma_hankel_planes_tc_run(ctypes.byref(prob), ctypes.byref(plan), og.data_ptr(), rg.data_ptr(),
                                                rh.data_ptr(), slot.data_ptr(), len(planes), pl.data_ptr(),
                                                tcs.data_ptr(), ntc, st), "mma_hankel_planes_tc_run")
            if _events is not None:
                _events[1].record(strm)
            if ff_planes:
                _check(lib.mma_hankel_ff_from_planes(ctypes.byref(prob), zg.data_ptr(), slot.data_ptr(), pl.data_ptr(),
                                                     ff.data_ptr(), st), "mma_hankel_ff_from_planes")
            _check(lib.mma_hankel_planes_tc_status(ctypes.byref(prob), ctypes.byref(plan), tcs.data_ptr(), st),
                   "mma_hankel_planes_tc (kernel status)")
        plan_d = plan.as_dict()
        plan_d["planes_via"] = ("tc" if use_tc else ("series" if len(planes) <= SERIES_PLANES else "direct")) \
            if planes else None
        plan_d["ff_via"] = "planes" if ff_planes else "fast"
    else:
        raise ValueError("form must be 'plain' or 'fast'")
    out_planes = {p: pl[i] for i, p in enumerate(planes)} if planes else {}
    return ff, out_planes, plan_d


def _np(a):
    return a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)


def _far_field_streamed(ogrid, rgrid, zgrid, rho, source, distance, pre_table, near_field, planes, tol, stream,
                        planes_via, ff_via):
    """far_field of a pinned host source [Nz, No, Nr]: blocks of STREAM_BLOCK frequencies are
    copied to the device on a second stream (mma_hankel_copy_block, one 2-D copy per block) and
    each block's fast form runs on `stream` as soon as its copy has landed, with the plan of the
    whole frequency range.  Returns once every block's copy has completed (the host source may
    then be released); the far field itself is ordered on `stream`."""
    lib = _sig()
    dev = torch.device("cuda", torch.cuda.current_device())
    comp = stream or torch.cuda.current_stream(dev)
    Nz, No, Nr = source.shape
    if len(zgrid) != Nz or len(ogrid) != No or len(rgrid) != Nr:
        raise ValueError("source shape does not match the grids")
    with torch.cuda.stream(comp):
        S = torch.empty(source.shape, dtype=source.dtype, device=dev)
        # the grids and the pre-factor first, as plain (synchronous) copies: they land before any
        # block is queued, and the blocks' calls take them from the device
        og, rg, zg, rh = (a.to(device=dev, dtype=torch.float64) if torch.is_tensor(a) else
                          torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
                          for a in (ogrid, rgrid, zgrid, rho))
        pre = None
        if pre_table is not None:
            pre = pre_table.to(device=dev, dtype=torch.complex128) if torch.is_tensor(pre_table) else \
                torch.as_tensor(np.ascontiguousarray(pre_table, dtype=np.complex128), device=dev)
    copy_s = torch.cuda.Stream(device=dev)
    copy_s.wait_stream(comp)  # S is allocated on comp
    S.record_stream(copy_s)
    esz = source.element_size()
    bounds = list(range(0, No, STREAM_BLOCK)) + [No]
    landed = []
    for a, b in zip(bounds[:-1], bounds[1:]):
        off = a * Nr * esz
        _check(lib.mma_hankel_copy_block(S.data_ptr() + off, source.data_ptr() + off, Nz, No * Nr * esz,
                                         (b - a) * Nr * esz, copy_s.cuda_stream), "mma_hankel_copy_block")
        ev = torch.cuda.Event()
        ev.record(copy_s)
        landed.append(ev)
    omax = float(np.max(np.abs(_np(ogrid))))
    ff = out_planes = plan = None
    with torch.cuda.stream(comp):
        for (a, b), ev in zip(zip(bounds[:-1], bounds[1:]), landed):
            comp.wait_event(ev)
            pre_b = None if pre is None else pre[:, a:b]
            ffb, plb, plan = far_field(og[a:b], rgrid, zgrid, rho, S[:, a:b], distance, pre_b, near_field, planes,
                                       form="fast", tol=tol, stream=comp, planes_via=planes_via, ff_via=ff_via,
                                       _omega_max=omax, _grids=(og[a:b], rg, zg, rh))
            if ff is None:
                ff = torch.empty(ffb.shape[0], No, dtype=ffb.dtype, device=dev)
                out_planes = {p: torch.empty(v.shape[0], No, dtype=v.dtype, device=dev) for p, v in plb.items()}
            ff[:, a:b] = ffb
            for p, v in plb.items():
                out_planes[p][:, a:b] = v
    landed[-1].synchronize()  # every block is on the device: the host source is no longer read
    return ff, out_planes, plan


class FarFieldPlan:
    """The fast form of far_field for one set of inputs, recorded once as a CUDA graph and replayed:
    the same kernels and the same result as far_field(..., form="fast"), without the host's work
    per call (the plan, the uploads of the grids, some ten launches).  The source and the
    pre-factor table stay on the device where they are; replay() recomputes from their current
    contents, so a new source of the same shape is copied into `source` before a replay.  Up to
    SERIES_PLANES requested planes (the entry and exit planes); more planes take far_field."""

    def __init__(self, ogrid, rgrid, zgrid, rho, source, distance, pre_table=None, near_field=True, planes=(),
                 tol=1e-9):
        if not source.is_cuda:
            raise ValueError("the source of a FarFieldPlan lives on the device")
        if len(set(planes)) > SERIES_PLANES:
            raise ValueError("a FarFieldPlan computes at most %d planes; far_field computes more" % SERIES_PLANES)
        dev = source.device
        self.source = source
        host = [np.ascontiguousarray(_np(a), dtype=np.float64) for a in (ogrid, rgrid, zgrid, rho)]
        self._grids = tuple(torch.as_tensor(a, device=dev) for a in host)  # kept: the graph reads them
        self.pre = None if pre_table is None else _dev(pre_table, dev, torch.complex128)
        kw = dict(pre_table=self.pre, near_field=near_field, planes=planes, form="fast", tol=tol,
                  planes_via="direct", _grids=self._grids)
        torch.cuda.synchronize(dev)
        s = torch.cuda.Stream(device=dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(s):  # one eager call first: the library's one-time state is made outside the capture
            far_field(*host, source, distance, stream=s, **kw)
        torch.cuda.current_stream(dev).wait_stream(s)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.ff, self.planes, self.plan = far_field(*host, source, distance, **kw)

    def replay(self):
        """Run the recorded far field on the current stream; returns (FF [Nrho, No], {plane: [Nrho, No]})."""
        self.graph.replay()
        return self.ff, self.planes


def HankelTransform(ogrid, rgrid, FField, distance, rgrid_FF, integrator=trapezoidal_integrator,
                    near_field_factor=True, pre_factor=1.0, form="plain"):
    """One plane (Hankel_transform.py:452-519): FField[omega, r] -> [omega, rho] complex128."""
    if integrator is not trapezoidal_integrator:
        raise NotImplementedError("only the trapezoidal radial integrator is implemented")
    pre = None
    pf = np.asarray(pre_factor)
    if pf.ndim == 2:  # pre_factor[r, omega] (:505-512)
        pre = pf[0][None, :] if np.all(pf == pf[:1, :]) else np.ascontiguousarray(pf.T)[None, :, :]
    elif pf.ndim == 0 and pf != 1.0:
        pre = np.full((1, len(ogrid)), complex(pf))
    src = FField if torch.is_tensor(FField) else torch.from_numpy(np.ascontiguousarray(FField))
    if src.dtype not in (torch.complex64, torch.complex128):
        src = src.to(torch.complex128)
    src = src.to("cuda")[None]
    # a single plane at z = 0 with the plane's own distance
    _, planes, _ = far_field(ogrid, rgrid, np.zeros(1), rgrid_FF, src, distance, pre, near_field_factor, planes=(0,),
                             form=form)
    return planes[0].T.cpu().numpy()


class Hankel_long:
    """Longitudinally integrated far field (Hankel_transform.py:523-686)."""

    def __init__(self, target, distance, rgrid_FF, preset_gas="vacuum", pressure=1.0, absorption_tables="Henke",
                 include_absorption=True, dispersion_tables="Henke", include_dispersion=True,
                 effective_IR_refrective_index=1.0, integrator_Hankel=trapezoidal_integrator,
                 integrator_longitudinal="trapezoidal", near_field_factor=True, store_cumulative_result=False,
                 store_non_normalised_cumulative_result=False, store_entry_and_exit_plane_transform=True,
                 form="plain", tol=1e-9, as_numpy=True):
        if not (integrator_longitudinal == "trapezoidal"):
            raise NotImplementedError("only logitudinal trapezoidal integrator implemented so far")
        if integrator_Hankel is not trapezoidal_integrator:
            raise NotImplementedError("only the trapezoidal radial integrator is implemented")
        self.include_dispersion = include_dispersion
        if include_dispersion:
            self.dispersion_tables = dispersion_tables
        self.include_absorption = include_absorption
        if include_absorption:
            self.absorption_tables = absorption_tables
        self.effective_IR_refrective_index = effective_IR_refrective_index
        self.integrator_Hankel = integrator_Hankel
        self.integrator_longitudinal = integrator_longitudinal
        self.near_field_factor = near_field_factor
        self.rgrid = rgrid_FF
        self.ogrid = np.copy(target.ogrid)
        cum = store_cumulative_result or store_non_normalised_cumulative_result
        if cum:
            self.zgrid = np.copy(target.zgrid)
        if not (((preset_gas + "_" + absorption_tables in XUV_index.gases) and
                 (preset_gas + "_" + dispersion_tables in XUV_index.gases)) or (preset_gas == "vacuum")):
            raise ValueError("Wrongly specified preset gas (or tables).")
        if store_cumulative_result and isinstance(pressure, dict) and "rgrid" in pressure:
            raise NotImplementedError("Renormalisation of the signal is not implemented for radially modulated density.")
        pre, renorm = pre_factor_table(target.zgrid, target.ogrid, preset_gas, pressure, absorption_tables,
                                       include_absorption, dispersion_tables, include_dispersion,
                                       effective_IR_refrective_index, rgrid=target.rgrid)
        z = np.asarray(target.zgrid, dtype=np.float64)
        Nz = len(z)
        if Nz < 2:
            raise ValueError("Hankel_long needs at least two source planes")
        want = set()
        if store_entry_and_exit_plane_transform:
            want |= {0, Nz - 1}
        if cum:
            want |= set(range(Nz))
        ff, planes, plan = far_field(target.ogrid, target.rgrid, z, rgrid_FF, target.source, distance, pre,
                                     near_field_factor, planes=sorted(want), form=form, tol=tol)
        self.fast_plan = plan
        conv = (lambda t: t.cpu().numpy()) if as_numpy else (lambda t: t)
        self.FF_integrated = conv(ff)
        if store_entry_and_exit_plane_transform:
            self.entry_plane_transform = conv(planes[0])
            self.exit_plane_transform = conv(planes[Nz - 1])
        if cum:
            P = torch.stack([planes[k] for k in range(Nz)])  # [Nz, Nrho, No]
            dz = torch.as_tensor(np.diff(z), device=P.device, dtype=torch.float64)
            contrib = 0.5 * dz[:, None, None] * (P[:-1] + P[1:])
            run = torch.cumsum(contrib, dim=0)  # running z-trapezoid after planes 1..Nz-1
            if store_cumulative_result:
                rn = torch.as_tensor(renorm[:Nz - 1], device=P.device)
                self.cumulative_field = conv(rn[:, None, :] * run)  # renorm_factor(k1), :668
            if store_non_normalised_cumulative_result:
                self.cumulative_field_no_norm = conv(run)


def Signal_cum_integrator(ogrid, zgrid, FSourceTerm, integrator=None):
    """Cumulative trapezoid of FSourceTerm[omega, z] along z (Hankel_transform.py:691-698)."""
    z = torch.as_tensor(np.asarray(zgrid, dtype=np.float64), device="cuda")
    F = torch.as_tensor(np.asarray(FSourceTerm), device="cuda").to(torch.complex128)
    out = torch.zeros_like(F)
    out[:, 1:] = torch.cumsum(0.5 * (z[1:] - z[:-1])[None, :] * (F[:, 1:] + F[:, :-1]), dim=1)
    return out.cpu().numpy()
