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

``save_to_hdf5`` / ``load_from_hdf5`` keep the reference's archive layout
(``TDSE_inputs/*``, ``TDSE_outputs/*``, float32 and int32 as it stores them,
PythonCTDSE/structures.py:133-166, 301-340, 454-532) through the package's own HDF5 module
(mma_gb300.h5io).  Arrays loaded from an archive are owned by the Python record (kept alive on
it), not by the library: do not pass such a record to the destructors.
"""
import ctypes
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

    def get_tgrid(self):
        return as_array(self.Efield.tgrid, self.Efield.Nt)

    def get_Efield(self):
        return as_array(self.Efield.Field, self.Efield.Nt)

    def init_time_and_field(self, DLL, filename="", z_i=0, r_i=0, E=None, t=None):
        """Time grid and field from arrays (E, t) or from a macroscopic archive
        (structures.py:242-299): CUPRAD/outputs/tgrid / TIMEau and output_field[z_i, :, r_i] /
        EFIELDau, the [z, t, r] order the MPI driver reads (MPI-TDSE.c:185).  The library copies
        the arrays (set_time_and_field)."""
        if filename != "" and (E is None or t is None):
            from . import h5io
            from .archive import EFIELDau, TIMEau

            with h5io.File(filename) as f:
                fld = f["CUPRAD/outputs/output_field"]
                if not 0 <= z_i < fld.shape[0]:
                    raise IndexError("z index %d outside 0..%d" % (z_i, fld.shape[0] - 1))
                if not 0 <= r_i < fld.shape[2]:
                    raise IndexError("r index %d outside 0..%d" % (r_i, fld.shape[2] - 1))
                t = np.asarray(f["CUPRAD/outputs/tgrid"][()], dtype=np.float64) / TIMEau
                E = np.asarray(fld[()][z_i, :, r_i], dtype=np.float64) / EFIELDau
        t = np.ascontiguousarray(t, dtype=np.float64)
        E = np.ascontiguousarray(E, dtype=np.float64)
        if len(t) != len(E):
            raise ValueError("time and field arrays differ in length")
        self.Efield.Nt = len(t)
        DLL.set_time_and_field(self.ptr, t, E, len(t))

    def save_to_hdf5(self, filename):
        """Append the inputs to ``filename`` under TDSE_inputs/ (structures.py:301-340): the
        scalars always; field and time grid once set; ground state, x grid and Einit once the
        ground state is computed.  Existing datasets are left as they are."""
        from . import h5io

        f = h5io.File(filename, "a")
        g = f.require_group("TDSE_inputs")
        items = [("trg_a", "f4", self.trg.a), ("dx", "f4", self.dx), ("dt", "f4", self.dt),
                 ("Eguess", "f4", self.Eguess), ("N_r_grid", "i4", self.num_r), ("gauge_type", "i4", self.gauge),
                 ("Ntinterp", "i4", self.Ntinterp), ("InterpByDTorNT", "i4", self.InterpByDTorNT),
                 ("analy_writewft", "i4", self.analy.writewft), ("analy_tprint", "f4", self.analy.tprint),
                 ("CV_criterion_of_GS", "f4", self.CV), ("x_int", "f4", self.x_int), ("num_t", "i4", self.num_t)]
        if self.Efield.Nt != 0:
            items += [("Nt", "i4", self.Efield.Nt), ("Efield", "f4", self.get_Efield()),
                      ("tgrid", "f4", self.get_tgrid())]
        if self.Einit != 0.0:
            gs = self.get_GS()
            items += [("psi0", "f4", np.stack([gs.real, gs.imag], axis=1)), ("x_grid", "f4", self.get_xgrid()),
                      ("Einit", "f4", self.Einit)]
        for name, dt, v in items:
            if name not in g:
                g.create_dataset(name, dtype=dt, data=v)
        f.close()

    def load_from_hdf5(self, filename):
        """Scalars, and where present the grid, ground state and field, from TDSE_inputs/
        (structures.py:133-166); precision is set to 'd'."""
        from . import h5io

        with h5io.File(filename) as f:
            g = f["TDSE_inputs"]
            self.Eguess = float(g["Eguess"][()])
            self.num_r = int(g["N_r_grid"][()])
            self.dx = float(g["dx"][()])
            self.InterpByDTorNT = int(g["InterpByDTorNT"][()])
            self.dt = float(g["dt"][()])
            self.Ntinterp = int(g["Ntinterp"][()])
            self.analy.writewft = int(g["analy_writewft"][()])
            self.analy.tprint = float(g["analy_tprint"][()])
            self.x_int = float(g["x_int"][()])
            self.trg.a = float(g["trg_a"][()])
            self.CV = float(g["CV_criterion_of_GS"][()])
            self.gauge = int(g["gauge_type"][()])
            self.precision = b"d"
            self._owned = getattr(self, "_owned", {})
            if "x_grid" in g and "psi0" in g and "Einit" in g:
                self._owned["x"] = _owned_array(g["x_grid"][()], self.num_r + 1)
                self._owned["psi0"] = _owned_array(np.asarray(g["psi0"][()]).reshape(-1), 2 * (self.num_r + 1))
                self.x = self._owned["x"].ctypes.data_as(POINTER(c_double))
                self.psi0 = self._owned["psi0"].ctypes.data_as(POINTER(c_double))
                self.Einit = float(g["Einit"][()])
            if "Nt" in g and "Efield" in g and "tgrid" in g:
                self.Efield.Nt = int(g["Nt"][()])
                self._owned["Field"] = _owned_array(g["Efield"][()], self.Efield.Nt)
                self._owned["tgrid"] = _owned_array(g["tgrid"][()], self.Efield.Nt)
                self.Efield.Field = self._owned["Field"].ctypes.data_as(POINTER(c_double))
                self.Efield.tgrid = self._owned["tgrid"].ctypes.data_as(POINTER(c_double))


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

    def get_wavefunction(self, inputs, grids=True):
        """Snapshots stored when ``inputs.analy.writewft`` is set, as a complex
        [n_snap, num_r+1] array (same count rule as prop.c:59-64); with ``grids`` (the
        reference's default, structures.py:548-584) returns (tgrid, x, wavefunction), the
        snapshot times spread evenly over the output time grid as the reference spreads them."""
        if not inputs.analy.writewft or not self.psi:
            return None
        t = self.get_tgrid()
        steps = int(np.floor(inputs.analy.tprint / (t[1] - t[0])))
        n_snap = int(self.Nt // steps)
        rows = getattr(self, "_owned", {}).get("psi_rows")
        if rows is not None:  # loaded from an archive: only the stored rows exist
            n_snap = min(n_snap, len(rows))
        n = inputs.num_r + 1
        wf = np.stack([as_complex(self.psi[i], n) for i in range(n_snap)]) if n_snap else None
        if not grids:
            return wf
        tg = np.array([t[self.Nt - 1]]) if n_snap == 1 else np.linspace(t[0], t[-1], n_snap)
        return tg, inputs.get_xgrid(), wf

    def save_to_hdf5(self, filename, inputs=None):
        """Append the outputs to ``filename`` under TDSE_outputs/ (structures.py:454-505), with
        the snapshots as psi_re / psi_im when ``inputs`` is given and they were stored."""
        from . import h5io

        f = h5io.File(filename, "a")
        g = f.require_group("TDSE_outputs")
        fe, fs = self.get_FEfield(), self.get_Fsourceterm()
        items = [("Nomega", "i4", self.Nomega), ("Nt", "i4", self.Nt), ("tgrid", "f4", self.get_tgrid()),
                 ("Efield", "f4", self.get_Efield()), ("sourceterm", "f4", self.get_sourceterm()),
                 ("omegagrid", "f4", self.get_omegagrid()), ("FEfield", "f4", np.stack([fe.real, fe.imag], axis=1)),
                 ("Fsourceterm", "f4", np.stack([fs.real, fs.imag], axis=1)), ("PopTot", "f4", self.get_PopTot()),
                 ("PopInt", "f4", self.get_PopInt()), ("expval", "f4", self.get_expval())]
        if inputs is not None:
            wf = self.get_wavefunction(inputs, grids=False)
            if wf is not None:
                items += [("psi_re", "f4", wf.real), ("psi_im", "f4", wf.imag)]
        for name, dt, v in items:
            if name not in g:
                g.create_dataset(name, dtype=dt, data=v)
        f.close()

    def load_from_hdf5(self, filename):
        """The arrays of TDSE_outputs/ (structures.py:507-545), snapshots included when stored."""
        from . import h5io

        with h5io.File(filename) as f:
            g = f["TDSE_outputs"]
            self.Nomega = int(g["Nomega"][()])
            self.Nt = int(g["Nt"][()])
            own = self._owned = {}
            for name, n in (("tgrid", self.Nt), ("Efield", self.Nt), ("sourceterm", self.Nt), ("expval", self.Nt),
                            ("omegagrid", self.Nomega), ("PopTot", self.Nt), ("PopInt", self.Nt),
                            ("FEfield", 2 * self.Nomega), ("Fsourceterm", 2 * self.Nomega)):
                own[name] = _owned_array(np.asarray(g[name][()]).reshape(-1), n)
                setattr(self, name, own[name].ctypes.data_as(POINTER(c_double)))
            if "psi_re" in g and "psi_im" in g:
                re, im = np.asarray(g["psi_re"][()], np.float64), np.asarray(g["psi_im"][()], np.float64)
                rows = [np.ascontiguousarray(np.stack([r, i], axis=1).reshape(-1)) for r, i in zip(re, im)]
                own["psi_rows"] = rows
                own["psi"] = (POINTER(c_double) * len(rows))(*[r.ctypes.data_as(POINTER(c_double)) for r in rows])
                self.psi = ctypes.cast(own["psi"], POINTER(POINTER(c_double)))


def _owned_array(v, n):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
    if a.size != n:
        raise ValueError("archive array of %d values where %d are expected" % (a.size, n))
    return a


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
