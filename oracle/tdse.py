"""ctypes binding of the C restatement of the reference TDSE (test infrastructure).

``ground_state`` and ``propagate`` return plain numpy arrays; they follow the
reference's Initialise_grid_and_ground_state (1DTDSE/sources/tools.c:31-51) and
call1DTDSE (1DTDSE/sources/singleTDSE.c:28-117) -- see tdse_oracle.c for the
line-by-line map.
"""
import ctypes
from ctypes import POINTER, Structure, c_double, c_int

import numpy as np

from . import oracle_lib_path

_dp = POINTER(c_double)


class _Args(Structure):
    _fields_ = [
        ("num_r", c_int),
        ("dx", c_double),
        ("trg_a", c_double),
        ("x_int", c_double),
        ("x", _dp),
        ("psi0", _dp),
        ("n_field", c_int),
        ("tgrid_f", _dp),
        ("field_f", _dp),
        ("dt_req", c_double),
        ("interp_by_dt_or_nt", c_int),
        ("ntinterp", c_int),
        ("tmin", c_double),
        ("writewft", c_int),
        ("tprint", c_double),
    ]


class _Result(Structure):
    _fields_ = [
        ("tgrid", _dp),
        ("efield", _dp),
        ("sourceterm", _dp),
        ("poptot", _dp),
        ("popint", _dp),
        ("expval", _dp),
        ("omegagrid", _dp),
        ("fsource", _dp),
        ("fsource_m2", _dp),
        ("fefield", _dp),
        ("fefield_m2", _dp),
        ("psi_final", _dp),
        ("psi_snap", _dp),
        ("n_out", c_int),
        ("n_omega", c_int),
        ("k1", c_int),
        ("n_snap", c_int),
        ("dt", c_double),
    ]


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        lib = ctypes.CDLL(oracle_lib_path())
        lib.oracle_ground_state.argtypes = [c_int, c_double, c_double, c_double, c_double, c_int, _dp, _dp,
                                            POINTER(c_double), POINTER(c_int)]
        lib.oracle_ground_state.restype = c_int
        lib.oracle_tdse_sizes.argtypes = [c_int, _dp, c_double, c_int, c_int, POINTER(c_int), POINTER(c_double),
                                          POINTER(c_int), POINTER(c_int)]
        lib.oracle_tdse_sizes.restype = c_int
        lib.oracle_propagate.argtypes = [POINTER(_Args), POINTER(_Result)]
        lib.oracle_propagate.restype = c_int
        _LIB = lib
    return _LIB


def _p(a):
    return a.ctypes.data_as(_dp)


def ground_state(num_r, dx, trg_a, Eguess=-1.0, CV=1e-15, max_iter=1000):
    """Returns (x, psi0 complex128, Einit, iterations)."""
    n = num_r + 1
    x = np.zeros(n)
    psi = np.zeros(2 * n)
    e = c_double()
    it = c_int()
    st = _lib().oracle_ground_state(num_r, dx, trg_a, Eguess, CV, max_iter, _p(x), _p(psi), ctypes.byref(e),
                                    ctypes.byref(it))
    if st != 0:
        raise RuntimeError("oracle ground state failed with status %d" % st)
    return x, psi[0::2] + 1j * psi[1::2], e.value, it.value


def sizes(tgrid_f, dt_req=0.25, interp_by_dt_or_nt=0, ntinterp=1):
    tg = np.ascontiguousarray(tgrid_f, dtype=np.float64)
    k1, dt, n_out, n_om = c_int(), c_double(), c_int(), c_int()
    st = _lib().oracle_tdse_sizes(len(tg), _p(tg), dt_req, interp_by_dt_or_nt, ntinterp, ctypes.byref(k1),
                                  ctypes.byref(dt), ctypes.byref(n_out), ctypes.byref(n_om))
    if st != 0:
        raise ValueError("bad time grid")
    return k1.value, dt.value, n_out.value, n_om.value


def propagate(x, psi0, tgrid_f, field_f, dx, trg_a, x_int=2.0, dt_req=0.25, interp_by_dt_or_nt=0, ntinterp=1,
              tmin=0.0, writewft=0, tprint=10.0):
    """Run one TDSE instance; returns a dict of numpy arrays keyed like the
    reference outputs (sourceterm, PopTot, PopInt, expval, Efield, tgrid,
    omegagrid, Fsourceterm, FsourcetermM2, FEfield, FEfieldM2, psi, snapshots)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = len(x)
    psi_il = np.empty(2 * n)
    psi_il[0::2] = np.real(psi0)
    psi_il[1::2] = np.imag(psi0)
    tg = np.ascontiguousarray(tgrid_f, dtype=np.float64)
    fl = np.ascontiguousarray(field_f, dtype=np.float64)
    k1, dt, n_out, n_om = sizes(tg, dt_req, interp_by_dt_or_nt, ntinterp)
    ts = {k: np.zeros(n_out + 1) for k in ("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval")}
    om = np.zeros(n_om)
    fs, fe = np.zeros(2 * n_om), np.zeros(2 * n_om)
    fsm, fem = np.zeros(n_om), np.zeros(n_om)
    psi_f = np.zeros(2 * n)
    n_snap = 0
    if writewft:
        n_snap = n_out // int(np.floor(tprint / dt))
    snaps = np.zeros(max(n_snap, 1) * 2 * n)
    a = _Args(n - 1, dx, trg_a, x_int, _p(x), _p(psi_il), len(tg), _p(tg), _p(fl), dt_req, interp_by_dt_or_nt,
              ntinterp, tmin, writewft, tprint)
    r = _Result(_p(ts["tgrid"]), _p(ts["Efield"]), _p(ts["sourceterm"]), _p(ts["PopTot"]), _p(ts["PopInt"]),
                _p(ts["expval"]), _p(om), _p(fs), _p(fsm), _p(fe), _p(fem), _p(psi_f), _p(snaps))
    st = _lib().oracle_propagate(ctypes.byref(a), ctypes.byref(r))
    if st != 0:
        raise RuntimeError("oracle propagate failed with status %d" % st)
    out = {k: v[:n_out] for k, v in ts.items()}
    out.update(omegagrid=om, Fsourceterm=fs[0::2] + 1j * fs[1::2], FsourcetermM2=fsm,
               FEfield=fe[0::2] + 1j * fe[1::2], FEfieldM2=fem, psi=psi_f[0::2] + 1j * psi_f[1::2],
               n_out=n_out, n_omega=n_om, k1=k1, dt=dt)
    if n_snap:
        s = snaps.reshape(n_snap, 2 * n)
        out["snapshots"] = s[:, 0::2] + 1j * s[:, 1::2]
    return out
