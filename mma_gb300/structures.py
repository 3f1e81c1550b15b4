"""ctypes mirrors of the TDSE parameter and result records.

These are the records the reference DLL exchanges with its Python host
(1DTDSE/sources/structures.h:16-147, mirrored on the Python side in
1DTDSE/PythonCTDSE/structures.py:18-56,110-131,437-452).  Field order, types and
therefore byte layout must match exactly: the GPU library exports the same
legacy symbols (``Initialise_grid_and_ground_state``, ``call1DTDSE``, ...) and
reads/writes these records in place, so either DLL can be driven by the same
host code.  Only the layout is shared with the reference; the helpers below
(numpy views instead of element-by-element copies, a default-parameter setter)
are this package's own.
"""
from ctypes import (
    POINTER,
    Structure,
    byref,
    c_char,
    c_double,
    c_int,
)

import numpy as np


class Efield_var(Structure):
    """Sampled driving field (structures.h:16-33)."""

    _fields_ = [
        ("tgrid", POINTER(c_double)),
        ("Field", POINTER(c_double)),
        ("dt", c_double),
        ("omega", c_double),
        ("E0", c_double),
        ("phi", c_double),
        ("ton", c_double),
        ("toff", c_double),
        ("Nt", c_int),
        ("nc", c_int),
    ]


class trg_def(Structure):
    """Soft-Coulomb target: V(x) = -1/sqrt(a^2 + x^2) (structures.h:39-42)."""

    _fields_ = [("a", c_double)]


class analy_def(Structure):
    """Wavefunction snapshot controls (structures.h:48-53)."""

    _fields_ = [("tprint", c_double), ("writewft", c_int)]


class output_print_def(Structure):
    """Output selection flags (structures.h:59-71)."""

    _fields_ = [
        ("Efield", c_int),
        ("FEfield", c_int),
        ("sourceterm", c_int),
        ("Fsourceterm", c_int),
        ("FEfieldM2", c_int),
        ("FsourceTermM2", c_int),
        ("PopTot", c_int),
        ("tgrid", c_int),
        ("omegagrid", c_int),
        ("PopInt", c_int),
        ("expval_x", c_int),
    ]


class inputs_def(Structure):
    """TDSE inputs (structures.h:80-118).

    The library allocates ``x`` and ``psi0`` in ``Initialise_grid_and_ground_state``
    and ``Efield.tgrid``/``Efield.Field`` in ``set_time_and_field``; release them
    with ``inputs_destructor`` exactly once.
    """

    _fields_ = [
        ("trg", trg_def),
        ("Efield", Efield_var),
        ("Eguess", c_double),
        ("Einit", c_double),
        ("tmin", c_double),
        ("Nt", c_int),
        ("num_t", c_int),
        ("dt", c_double),
        ("num_r", c_int),
        ("dx", c_double),
        ("psi0", POINTER(c_double)),
        ("x", POINTER(c_double)),
        ("gauge", c_int),
        ("x_int", c_double),
        ("analy", analy_def),
        ("InterpByDTorNT", c_int),
        ("Ntinterp", c_int),
        ("Print", output_print_def),
        ("CV", c_double),
        ("precision", c_char * 2),
    ]

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        self.ptr = byref(self)

    def init_default_inputs(self, Eguess=-1.0, num_r=16000, dx=0.4, InterpByDTorNT=0, dt=0.25,
                            trg_a=1.3677, CV=1e-25, gauge=0, Ntinterp=1, writewft=0, tprint=10.0,
                            x_int=2.0, precision=b"d"):
        """Set the scalar inputs; the defaults are the reference's Python defaults
        (PythonCTDSE/structures.py:176-237)."""
        self.Eguess = Eguess
        self.num_r = num_r
        self.dx = dx
        self.InterpByDTorNT = InterpByDTorNT
        self.dt = dt
        self.Ntinterp = Ntinterp
        self.analy.writewft = writewft
        self.analy.tprint = tprint
        self.x_int = x_int
        self.trg.a = trg_a
        self.CV = CV
        self.gauge = gauge
        self.precision = precision

    def get_xgrid(self):
        return as_array(self.x, self.num_r + 1)

    def get_GS(self):
        return as_complex(self.psi0, self.num_r + 1)


class outputs_def(Structure):
    """TDSE results (structures.h:120-147).  Arrays are allocated by ``call1DTDSE``;
    release them with ``outputs_destructor`` exactly once."""

    _fields_ = [
        ("tgrid", POINTER(c_double)),
        ("Efield", POINTER(c_double)),
        ("sourceterm", POINTER(c_double)),
        ("omegagrid", POINTER(c_double)),
        ("FEfield", POINTER(c_double)),
        ("Fsourceterm", POINTER(c_double)),
        ("FEfieldM2", POINTER(c_double)),
        ("FsourcetermM2", POINTER(c_double)),
        ("PopTot", POINTER(c_double)),
        ("PopInt", POINTER(c_double)),
        ("expval", POINTER(c_double)),
        ("Nt", c_int),
        ("Nomega", c_int),
        ("psi", POINTER(POINTER(c_double))),
    ]

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        self.ptr = byref(self)

    def get_tgrid(self):
        return as_array(self.tgrid, self.Nt)

    def get_Efield(self):
        return as_array(self.Efield, self.Nt)

    def get_sourceterm(self):
        return as_array(self.sourceterm, self.Nt)

    def get_PopTot(self):
        return as_array(self.PopTot, self.Nt)

    def get_PopInt(self):
        return as_array(self.PopInt, self.Nt)

    def get_expval(self):
        return as_array(self.expval, self.Nt)

    def get_omegagrid(self):
        return as_array(self.omegagrid, self.Nomega)

    def get_Fsourceterm(self):
        return as_complex(self.Fsourceterm, self.Nomega)

    def get_FEfield(self):
        return as_complex(self.FEfield, self.Nomega)

    def get_FsourcetermM2(self):
        return as_array(self.FsourcetermM2, self.Nomega)

    def get_FEfieldM2(self):
        return as_array(self.FEfieldM2, self.Nomega)

    def get_wavefunction(self, inputs):
        """Snapshots stored when ``inputs.analy.writewft`` is set, as a complex
        [n_snap, num_r+1] array (same count rule as prop.c:59-64)."""
        if not inputs.analy.writewft or not self.psi:
            return None
        t = self.get_tgrid()
        steps = int(np.floor(inputs.analy.tprint / (t[1] - t[0])))
        n_snap = int(self.Nt // steps)
        n = inputs.num_r + 1
        return np.stack([as_complex(self.psi[i], n) for i in range(n_snap)]) if n_snap else None


def as_array(ptr, n):
    """Copy ``n`` doubles behind a ctypes pointer into a numpy array."""
    if not ptr or n <= 0:
        return np.zeros(0)
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def as_complex(ptr, n):
    """Copy ``n`` interleaved (re, im) pairs behind a ctypes pointer into complex128."""
    if not ptr or n <= 0:
        return np.zeros(0, dtype=np.complex128)
    flat = np.ctypeslib.as_array(ptr, shape=(2 * n,))
    return flat[0::2] + 1j * flat[1::2]
