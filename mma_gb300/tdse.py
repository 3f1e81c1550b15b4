"""Drop-in host class for the TDSE C-ABI (mirrors 1DTDSE/PythonTDSE.py:18-220).

``TDSE_DLL(path)`` binds a shared library that exports the reference DLL's
legacy symbols -- ``Initialise_grid_and_ground_state``, ``call1DTDSE``,
``set_time_and_field``, ``Set_all_prints``, ``inputs_destructor``,
``outputs_destructor``, ``free_arr``, ``free_mtrx``, ``window_analysis``,
``GaborTransform`` -- with the record layouts of
``mma_gb300.structures``.  With no path it binds this package's GPU library,
whose legacy symbols run the CUDA kernels.  The same class drives the reference
DLL built from its own sources, which is how the parity tests and the CPU
baseline call it.

Error behaviour: the reference prints and continues or calls exit(); the GPU
library never exits -- its legacy entry points record a status readable through
``mma_last_error``/``mma_last_error_message`` and this class raises
``MMAError`` when that status is non-zero.
"""
import ctypes
from ctypes import CDLL, POINTER, c_double, c_int

import numpy as np

from .structures import inputs_def, output_print_def, outputs_def


class MMAError(RuntimeError):
    pass


class TDSE_DLL:
    def __init__(self, path_to_DLL=None):
        if path_to_DLL is None:
            from ._lib import lib_path

            path_to_DLL = lib_path()
        self.path = path_to_DLL
        self.DLL = CDLL(path_to_DLL)
        d = self.DLL
        d.Initialise_grid_and_ground_state.restype = None
        d.Initialise_grid_and_ground_state.argtypes = [POINTER(inputs_def)]
        d.call1DTDSE.restype = None
        d.call1DTDSE.argtypes = [POINTER(inputs_def), POINTER(outputs_def)]
        d.set_time_and_field.restype = None
        d.set_time_and_field.argtypes = [POINTER(inputs_def), POINTER(c_double), POINTER(c_double), c_int]
        d.inputs_destructor.restype = None
        d.inputs_destructor.argtypes = [POINTER(inputs_def)]
        d.outputs_destructor.restype = None
        d.outputs_destructor.argtypes = [POINTER(outputs_def)]
        d.free_arr.restype = None
        d.free_arr.argtypes = [POINTER(c_double)]
        d.free_mtrx.restype = None
        d.free_mtrx.argtypes = [POINTER(POINTER(c_double)), c_int]
        d.Set_all_prints.restype = output_print_def
        d.Set_all_prints.argtypes = []
        self._has_status = hasattr(d, "mma_last_error")
        if self._has_status:
            d.mma_last_error.restype = c_int
            d.mma_last_error.argtypes = []
            d.mma_last_error_message.restype = ctypes.c_char_p
            d.mma_last_error_message.argtypes = []

    def _check(self, what):
        if self._has_status:
            st = self.DLL.mma_last_error()
            if st != 0:
                msg = self.DLL.mma_last_error_message().decode(errors="replace")
                raise MMAError("%s failed (status %d): %s" % (what, st, msg))

    def init_GS(self, inputs):
        """Grid and ground state (tools.c:31-51): allocates ``inputs.x`` and ``inputs.psi0``."""
        self.DLL.Initialise_grid_and_ground_state(inputs.ptr)
        self._check("Initialise_grid_and_ground_state")

    def call1DTDSE(self, inputs, outputs):
        """Propagate the ground state through ``inputs.Efield`` (singleTDSE.c:28-117)."""
        self.DLL.call1DTDSE(inputs.ptr, outputs.ptr)
        self._check("call1DTDSE")

    def set_time_and_field(self, in_ptr, time, field, N):
        t = np.ascontiguousarray(time, dtype=np.float64)
        f = np.ascontiguousarray(field, dtype=np.float64)
        self.DLL.set_time_and_field(in_ptr, t.ctypes.data_as(POINTER(c_double)),
                                    f.ctypes.data_as(POINTER(c_double)), int(N))

    def init_prints(self, inputs):
        inputs.Print = self.DLL.Set_all_prints()

    def compute_PES(self, inputs, psi, E_start=-0.6, num_E=10000, epsilon=5e-4, Estep=5e-4):
        """Photoelectron spectrum of ``psi`` by the resolvent window method
        (window_analysis, tools.c:206-316; PythonTDSE.py:80-109): returns (E_grid, PES).
        ``psi``: complex numpy array of num_r + 1 values or a ctypes pointer to interleaved
        doubles.  ``inputs`` supplies num_r, dx and trg.a (passed by value)."""
        f = self.DLL.window_analysis
        f.restype = POINTER(c_double)
        f.argtypes = [inputs_def, POINTER(c_double), c_int, c_double, c_double, c_double]
        if isinstance(psi, np.ndarray):
            il = np.empty(2 * len(psi))
            il[0::2] = np.real(psi)
            il[1::2] = np.imag(psi)
            ptr = il.ctypes.data_as(POINTER(c_double))
        else:
            il, ptr = None, psi
        res = f(inputs, ptr, int(num_E), float(epsilon), float(Estep), float(E_start))
        self._check("window_analysis")
        if not res:
            raise MMAError("window_analysis returned no result")
        out = np.ctypeslib.as_array(res, shape=(int(num_E),)).copy()
        self.free_arr(res)
        return np.linspace(E_start, E_start + (num_E - 1) * Estep, num_E), out

    def gabor_transform(self, signal, dt, N, omega_max, t_min, t_max, N_G, a=8.0):
        """|Gabor transform| of ``signal`` (GaborTransform, tools_fftw3.c:158-213;
        PythonTDSE.py:111-150): returns (t grid [N_G], omegas [N_freq], |G| [N_freq, N_G]),
        with the frequencies 2 pi fftfreq(N, dt) up to omega_max."""
        f = self.DLL.GaborTransform
        f.restype = POINTER(POINTER(c_double))
        f.argtypes = [POINTER(c_double), c_double, c_int, c_int, c_int, c_double, c_double, c_double]
        omegas = 2 * np.pi * np.fft.fftfreq(int(N), dt)[0:int(N) // 2]
        sel = omegas <= omega_max
        n_freq = int(np.count_nonzero(sel))
        sig = np.ascontiguousarray(signal, dtype=np.float64)
        res = f(sig.ctypes.data_as(POINTER(c_double)), float(dt), int(N), n_freq, int(N_G), float(t_min),
                float(t_max), float(a))
        self._check("GaborTransform")
        if not res:
            raise MMAError("GaborTransform returned no result")
        g = np.stack([np.ctypeslib.as_array(res[i], shape=(n_freq,)).copy() for i in range(int(N_G))])
        self.free_mtrx(res, int(N_G))
        return np.linspace(t_min, t_max, int(N_G)), omegas[sel], g.T

    def free_mtrx(self, buffer_ptr, N_rows):
        self.DLL.free_mtrx(buffer_ptr, int(N_rows))

    def free_arr(self, buffer_ptr):
        self.DLL.free_arr(buffer_ptr)

    def free_outputs(self, out_ptr):
        self.DLL.outputs_destructor(out_ptr)

    def free_inputs(self, in_ptr):
        self.DLL.inputs_destructor(in_ptr)


def init_time_and_field(dll, inputs, t, E):
    """Same as the reference's ``inputs_def.init_time_and_field(DLL, E=, t=)``
    (PythonCTDSE/structures.py:291-299): the library copies the arrays."""
    t = np.asarray(t, dtype=np.float64)
    E = np.asarray(E, dtype=np.float64)
    if len(t) != len(E):
        raise ValueError("time and field arrays differ in length")
    inputs.Efield.Nt = len(t)
    dll.set_time_and_field(inputs.ptr, t, E, len(t))


def run_single(dll, t, E, num_r=8000, dx=0.1, trg_a=np.sqrt(1.68), dt=0.25, Eguess=-1.0, CV=1e-15, x_int=2.0,
               writewft=0, tprint=10.0, InterpByDTorNT=0, Ntinterp=1):
    """Convenience: one full TDSE through the legacy ABI, results as numpy arrays.

    Follows the reference's notebook/test call sequence (1DTDSE/tests.py:10-50):
    defaults, field, ground state, propagation, getters, destructors.
    """
    inp = inputs_def()
    inp.init_default_inputs(Eguess=Eguess, num_r=num_r, dx=dx, dt=dt, trg_a=trg_a, CV=CV, x_int=x_int,
                            writewft=writewft, tprint=tprint, InterpByDTorNT=InterpByDTorNT, Ntinterp=Ntinterp)
    init_time_and_field(dll, inp, t, E)
    out = outputs_def()
    try:
        dll.init_GS(inp)
        res = {"x": inp.get_xgrid(), "psi0": inp.get_GS(), "Einit": inp.Einit}
        dll.call1DTDSE(inp, out)
        res.update(
            tgrid=out.get_tgrid(), Efield=out.get_Efield(), sourceterm=out.get_sourceterm(),
            PopTot=out.get_PopTot(), PopInt=out.get_PopInt(), expval=out.get_expval(),
            omegagrid=out.get_omegagrid(), Fsourceterm=out.get_Fsourceterm(),
            FsourcetermM2=out.get_FsourcetermM2(), FEfield=out.get_FEfield(), FEfieldM2=out.get_FEfieldM2(),
            Nt=out.Nt, Nomega=out.Nomega, dt=inp.Efield.dt, num_t=inp.num_t, Ntinterp=inp.Ntinterp,
        )
        if writewft:
            res["snapshots"] = out.get_wavefunction(inp, grids=False)
            steps = int(np.floor(tprint / (res["tgrid"][1] - res["tgrid"][0])))
            n_snap = int(out.Nt // steps)
            if n_snap and out.psi:
                dll.free_mtrx(out.psi, n_snap)
                out.psi = None
    finally:
        dll.free_outputs(out.ptr)
        dll.free_inputs(inp.ptr)
    return res
