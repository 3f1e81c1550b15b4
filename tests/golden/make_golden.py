"""Generate the golden fixtures in this directory from the reference itself.

TDSE fixtures: the reference DLL compiled unchanged from its sources
(1DTDSE/sources, see oracle/Makefile `ref`) driven through its own C-ABI by
mma_gb300.tdse.TDSE_DLL -- the same host class that drives the GPU library.

Hankel fixtures: the reference's Hankel/Hankel_transform.py imported from the
reference checkout, with two modules it imports but this path does not use
replaced in sys.modules: h5py (file I/O only) and XUV_refractive_index, whose
dispersion_function/beta_factor_ref return the constant complex index of the
synthetic medium (n = 1 - 1e-5 + 1e-7 i by default), and `gases`.

Analysis fixtures: the same reference DLL's window_analysis and GaborTransform exports,
driven by TDSE_DLL.compute_PES / gabor_transform.

Refractive-index fixture: the reference's shared_python/make_table.py and
XUV_refractive_index.py run unchanged on synthetic tables (xuv_tables/, written here) with an
in-memory stand-in for h5py.

Stored-result fixture: the reference's own regression archive 1DTDSE/ionization.h5 (written by
its save_to_hdf5, read by 1DTDSE/tests.py:50-88), read with mma_gb300.h5io and kept as
ionization_h5.npz: every dataset as stored (float32 / int32), the wavefunction snapshots
subsampled to every 7th.

Run from the repository root where the reference checkout exists:
    python tests/golden/make_golden.py --ref <reference checkout>
"""
import argparse
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from tdse_cases import A_CONFIG, sin2_pulse  # noqa: E402

# Cases: name -> (run_single kwargs, pulse kwargs).  All pulses start one sample after
# t = 0 so the reference's zero gate is decided by the field, not by FFT round-off.
TDSE_CASES = {
    "tdse_small": (dict(num_r=600, dx=0.4, trg_a=A_CONFIG), dict(n_cycles=2)),
    "tdse_medium": (dict(num_r=2000, dx=0.2, trg_a=A_CONFIG), dict(n_cycles=3)),
    # the parameters of the reference's own regression test (1DTDSE/tests.py:13-39)
    "tdse_reftest": (dict(num_r=8000, dx=0.4, trg_a=1.0), dict(n_cycles=4, E0=0.14, omega=0.07)),
    # field sampled at exactly 0.5 a.u. > dt = 0.25: Fourier interpolation with k1 = 3
    "tdse_interp": (dict(num_r=600, dx=0.4, trg_a=A_CONFIG), dict(n_cycles=2, dt=0.5, exact_dt=True)),
    "tdse_snapshots": (dict(num_r=600, dx=0.4, trg_a=1.0, writewft=1, tprint=10.0), dict(n_cycles=1.5)),
    # config 0 of the benchmark: a^2 = 1.68, x in [-400, 400], dx = 0.1, 10-cycle 800 nm pulse
    "tdse_config0": (dict(num_r=8000, dx=0.1, trg_a=A_CONFIG), dict(n_cycles=10)),
}


def make_tdse(ref_src, only=None):
    import oracle
    from mma_gb300.tdse import TDSE_DLL, run_single

    os.environ["MMA_REF_SRC"] = ref_src
    oracle.build(ref=True)
    dll = TDSE_DLL(oracle.ref_dll_path())
    for name, (kw, pk) in TDSE_CASES.items():
        if only and name not in only:
            continue
        t, E = sin2_pulse(skip_first=True, **pk)
        r = run_single(dll, t, E, CV=1e-15, **kw)
        out = dict(t=t, E=E, Einit=r["Einit"], psi0_re=np.real(r["psi0"]), x=r["x"],
                   sourceterm=r["sourceterm"], PopTot=r["PopTot"], PopInt=r["PopInt"], expval=r["expval"],
                   Efield=r["Efield"], tgrid=r["tgrid"], omegagrid=r["omegagrid"],
                   Fsourceterm=r["Fsourceterm"], FsourcetermM2=r["FsourcetermM2"], FEfield=r["FEfield"],
                   Nt=r["Nt"], Nomega=r["Nomega"], dt=r["dt"],
                   params=np.array([kw["num_r"], kw["dx"], kw["trg_a"]]))
        if "snapshots" in r and r["snapshots"] is not None:
            out["snapshots"] = r["snapshots"]
            out["tprint"] = kw["tprint"]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "Nt", r["Nt"], "Einit", r["Einit"])


def analysis_inputs(seed=0):
    """A synthetic wavefunction (ground-state-like core plus a boosted wavepacket, seeded) for
    the photoelectron spectrum and a chirped sin^2 pulse for the Gabor transform."""
    rng = np.random.default_rng(seed)
    num_r, dx = 800, 0.2
    x = np.arange(num_r + 1) * dx - 0.5 * num_r * dx
    psi = (np.exp(-np.abs(x)) + 0.3 * np.exp(-((x - 20.0) / 6.0) ** 2) * np.exp(1j * 0.9 * x)
           + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)) * np.exp(-(x / 30.0) ** 2))
    dt, N = 0.25, 1500
    t = dt * np.arange(N)
    sig = np.sin(np.pi * t / (N * dt)) ** 2 * np.cos(0.057 * t + 2e-4 * t ** 2) + 0.02 * rng.standard_normal(N)
    return num_r, dx, psi, dt, N, sig


def make_analysis(ref_src):
    """PES (window_analysis) and Gabor (GaborTransform) through the reference DLL's own exports."""
    import oracle
    from mma_gb300.structures import inputs_def
    from mma_gb300.tdse import TDSE_DLL

    os.environ["MMA_REF_SRC"] = ref_src
    oracle.build(ref=True)
    dll = TDSE_DLL(oracle.ref_dll_path())
    num_r, dx, psi, dt, N, sig = analysis_inputs()
    inp = inputs_def()
    inp.init_default_inputs(num_r=num_r, dx=dx, trg_a=A_CONFIG)
    pes_kw = dict(E_start=-0.7, num_E=300, epsilon=5e-3, Estep=5e-3)
    E, P = dll.compute_PES(inp, psi, **pes_kw)
    gab_kw = dict(omega_max=1.5, t_min=0.0, t_max=N * dt, N_G=64, a=8.0)
    tg, om, G = dll.gabor_transform(sig, dt, N, **gab_kw)
    np.savez_compressed(os.path.join(HERE, "analysis.npz"), num_r=num_r, dx=dx, trg_a=A_CONFIG, psi=psi,
                        E=E, PES=P, dt=dt, N=N, signal=sig, t_gabor=tg, omegas=om, gabor=G,
                        pes_kw=np.array([pes_kw["E_start"], pes_kw["num_E"], pes_kw["epsilon"], pes_kw["Estep"]]),
                        gab_kw=np.array([gab_kw["omega_max"], gab_kw["t_min"], gab_kw["t_max"], gab_kw["N_G"],
                                         gab_kw["a"]]))
    print("analysis: PES", P.shape, "max", P.max(), "Gabor", G.shape)


XUV_GASES = {"he": 2.0, "ne": 10.0, "ar": 18.0, "kr": 36.0, "xe": 54.0}


def write_xuv_tables(directory):
    """Synthetic scattering-factor tables (smooth functions of the photon energy, this file's
    own numbers) in the two text formats of the reference's table directory: Henke ``*.nff``
    (one header line; E [eV], f1, f2; f1 = -9999 where not listed) and NIST ``*_f1_NIST.txt`` /
    ``*_f2_NIST.txt`` (three header lines and a blank one; E [keV], f)."""
    os.makedirs(directory, exist_ok=True)
    E = np.geomspace(10.0, 200.0, 48)
    for g, Z in XUV_GASES.items():
        f1 = Z * (1.0 - np.exp(-E / 50.0)) + 0.3 * np.sin(E / 7.0)
        f1[E < 18.0] = -9999.0
        f2 = Z * np.exp(-E / 40.0) * (E / 30.0)
        with open(os.path.join(directory, g + ".nff"), "w") as f:
            f.write("E(eV)\tf1\tf2\n")
            for e, a, b in zip(E, f1, f2):
                f.write("%.4f\t%.6g\t%.6E\n" % (e, a, b))
        for which, val in (("f1", Z * (1.0 - np.exp(-E / 45.0)) - 0.2 * np.cos(E / 9.0)), ("f2", 1.1 * f2)):
            with open(os.path.join(directory, "%s_%s_NIST.txt" % (g, which)), "w") as f:
                f.write("synthetic table\n    E              %s\n   keV           e atom-1\n\n" % which)
                for e, v in zip(E, val):
                    f.write("%.6E  %.5E\n" % (1e-3 * e, v))


class _MemH5:
    """In-memory stand-in for the two h5py calls of the reference's table scripts: File(...) in
    write mode (create_group, create_dataset, attrs) records the archive, read mode serves it."""
    store = {}

    class Dataset:
        def __init__(self, data):
            self.data = np.asarray(data)
            self.attrs = {}

        def __getitem__(self, k):
            return self.data[k]

    class Group(dict):
        def create_dataset(self, name, data=None):
            d = _MemH5.Dataset(data)
            self[name] = d
            return d

    class File:
        def __init__(self, path, mode="r"):
            key = os.path.basename(path)
            if mode == "w":
                _MemH5.store[key] = {}
            self.data = _MemH5.store[key]

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def create_group(self, name):
            g = _MemH5.Group()
            self.data[name] = g
            return g

        def keys(self):
            return self.data.keys()

        def __getitem__(self, k):
            return self.data[k]


def make_xuv(ref_root):
    """Tabulated refractive index: the reference's make_table.py (text tables -> archive) and
    XUV_refractive_index.py (archive -> dispersion_function, beta_factor_ref), run unchanged on
    the synthetic tables committed in xuv_tables/ with the in-memory h5py stand-in."""
    import runpy
    import shutil
    import tempfile

    tables = os.path.join(HERE, "xuv_tables")
    write_xuv_tables(tables)
    mod = types.ModuleType("h5py")
    mod.File = _MemH5.File
    sys.modules["h5py"] = mod
    sp = os.path.join(ref_root, "shared_python")
    sys.path.insert(0, sp)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        shutil.copytree(tables, os.path.join(d, "XUV_tables"))
        os.chdir(d)
        try:
            runpy.run_path(os.path.join(sp, "make_table.py"), run_name="__main__")
        finally:
            os.chdir(cwd)
    sys.modules.pop("XUV_refractive_index", None)
    import XUV_refractive_index as XR

    omega = np.geomspace(20.0, 190.0, 9) * 1.602176565e-19 / 1.0545718e-34  # photon energies 20..190 eV
    out = dict(omega=omega, gases=np.array(sorted(XR.gases)))
    for g in sorted(XR.gases):
        out["disp_" + g] = np.array([XR.dispersion_function(w, 0.7, g, n_IR=1.0003) for w in omega])
        out["beta_" + g] = np.array([XR.beta_factor_ref(w, g) for w in omega])
    np.savez_compressed(os.path.join(HERE, "xuv_index.npz"), **out)
    print("xuv index:", sorted(XR.gases))


def import_reference_hankel(ref_root, n_xuv=complex(1 - 1e-5, 1e-7)):
    """Import Hankel_transform.py from the reference with the two stubs described above."""
    sys.modules["h5py"] = types.ModuleType("h5py")
    xuv = types.ModuleType("XUV_refractive_index")
    sys.path.insert(0, os.path.join(ref_root, "shared_python"))
    import units  # the reference's own unit module

    xuv.gases = ["Ar_Henke", "Ar_NIST"]
    # n = n0 + i beta (XUV_refractive_index.py:164-167): 1/v_IR - 1/v_XUV = (n_IR - n0)/c
    xuv.dispersion_function = lambda omega, pressure, gas, n_IR=1.0, **kw: \
        pressure * (n_IR - n_xuv.real) / units.c_light * np.ones_like(np.asarray(omega, dtype=float))
    xuv.beta_factor_ref = lambda omega, gas, **kw: n_xuv.imag * np.ones_like(np.asarray(omega, dtype=float))
    sys.modules["XUV_refractive_index"] = xuv
    sys.path.insert(0, os.path.join(ref_root, "Hankel"))
    import Hankel_transform as HT

    return HT, units


HANKEL_CASES = {
    # name: (No, Nr, Nz_planes, Nrho, gas, near_field, cumulative)
    "hankel_small": (6, 24, 5, 12, "Ar", True, True),
    "hankel_vacuum": (5, 20, 4, 10, "vacuum", True, False),
    "hankel_far_only": (4, 16, 4, 8, "Ar", False, True),
    # config-3 geometry at reduced size: 512 -> 64 radii, 256 -> 17 planes, 2048 -> 12 frequencies
    "hankel_config3_slice": (12, 64, 16, 32, "Ar", True, True),
}


def radial_pressure():
    """A medium modulated in z and r (a jet narrowing downstream): the pressure table of the
    reference's zr branch."""
    pz = np.linspace(-6e-3, 6e-3, 13)
    pr = np.linspace(0.0, 300e-6, 11)
    val = np.exp(-(pr[None, :] / (150e-6 * (1.0 + 40.0 * (pz[:, None] + 6e-3)))) ** 2) * (1.0 - 0.3 * pz[:, None] / 6e-3)
    return dict(zgrid=pz, rgrid=pr, value=val)


def make_hankel_radial(ref_root):
    """The reference's zr-branch pre-factor (Hankel_transform.py:302-399) on the
    hankel_config3_slice grids, for each plane: get_propagation_pre_factor_function(...)[0](kz)."""
    HT, units = import_reference_hankel(ref_root)
    No, Nr, Nz, Nrho = HANKEL_CASES["hankel_config3_slice"][:4]
    zgrid, rgrid, ogrid, rho, S = hankel_inputs(No, Nr, Nz, Nrho)
    press = radial_pressure()
    target = HT.FSources_provider(zgrid, rgrid, ogrid, data_source="static", FSource=S)
    pf, renorm = HT.get_propagation_pre_factor_function(target.zgrid, target.rgrid, target.ogrid, preset_gas="Ar",
                                                        pressure=press)
    pre = np.stack([pf(k) for k in range(len(target.zgrid))])  # [Nz, No, Nr] as the reference returns it
    np.savez_compressed(os.path.join(HERE, "prefactor_radial.npz"), zgrid=target.zgrid, rgrid=target.rgrid,
                        ogrid=target.ogrid, pressure_zgrid=press["zgrid"], pressure_rgrid=press["rgrid"],
                        pressure_value=press["value"], pre=pre, renorm_is_none=renorm is None,
                        n_xuv=np.array([1 - 1e-5, 1e-7]))
    print("hankel radial pre-factor", pre.shape)


def hankel_inputs(No, Nr, Nz, Nrho, seed=0):
    """Seeded synthetic source with config-3 structure at small size: Gaussian radial
    profile (50 um) times a comb of odd harmonics (11..41 of 800 nm, Lorentzian width
    0.3 omega0) with random phases, complex64 like the production source."""
    rng = np.random.default_rng(seed)
    omega0 = 0.057 / 2.4188843265857e-17
    zgrid = np.linspace(-5e-3, 5e-3, Nz + 1)  # +1: FSources_provider drops the last plane
    rgrid = np.linspace(0.0, 200e-6, Nr)
    ogrid = np.linspace(10 * omega0, 42 * omega0, No)
    rho = np.linspace(0.0, 5e-3, Nrho)
    q = np.arange(11, 42, 2)
    phases = rng.uniform(0, 2 * np.pi, size=(Nz + 1, len(q)))
    lor = 1.0 / (1.0 + ((ogrid[None, :] - q[:, None] * omega0) / (0.3 * omega0)) ** 2)
    comb = np.einsum("zq,qo->zo", np.exp(1j * phases), lor)
    prof = np.exp(-(rgrid / 50e-6) ** 2)
    S = (comb[:, :, None] * prof[None, None, :]).astype(np.complex64)
    S = S * (1.0 + 0.3 * rng.standard_normal(S.shape)).astype(np.float32)
    return zgrid, rgrid, ogrid, rho, S


def make_hankel(ref_root):
    HT, units = import_reference_hankel(ref_root)
    for name, (No, Nr, Nz, Nrho, gas, nff, cum) in HANKEL_CASES.items():
        zgrid, rgrid, ogrid, rho, S = hankel_inputs(No, Nr, Nz, Nrho)
        target = HT.FSources_provider(zgrid, rgrid, ogrid, data_source="static", FSource=S)
        vac = gas == "vacuum"  # the reference has no tables for vacuum: both factors off
        res = HT.Hankel_long(target, 1.0, rho, preset_gas=gas, pressure=1.0, near_field_factor=nff,
                             store_cumulative_result=cum, include_dispersion=not vac, include_absorption=not vac)
        out = dict(zgrid=zgrid, rgrid=rgrid, ogrid=ogrid, rho=rho, S=S, FF_integrated=res.FF_integrated,
                   entry=res.entry_plane_transform, exit=res.exit_plane_transform, distance=1.0,
                   gas=np.bytes_(gas), near_field=nff, n_xuv=np.array([1 - 1e-5, 1e-7]))
        if cum:
            out["cumulative"] = res.cumulative_field
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, res.FF_integrated.shape)


IONIZATION_SNAPSHOTS = slice(0, None, 7)


def make_ionization(ref_root):
    """Every dataset of 1DTDSE/ionization.h5 (TDSE_inputs/*, TDSE_outputs/*) as stored; keys are
    the archive paths with '/' replaced by '__'."""
    from mma_gb300 import h5io

    f = h5io.File(os.path.join(ref_root, "1DTDSE", "ionization.h5"))
    out = {}
    for grp in ("TDSE_inputs", "TDSE_outputs"):
        for k in f[grp].keys():
            v = f[grp + "/" + k][()]
            if k in ("psi_re", "psi_im"):
                out["snapshot_index"] = np.arange(v.shape[0])[IONIZATION_SNAPSHOTS]
                v = v[IONIZATION_SNAPSHOTS]
            out[grp + "__" + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "ionization_h5.npz"), **out)
    print("ionization_h5", len(out), "arrays")


LAYOUT_STRUCTS = ["Efield_var", "trg_def", "analy_def", "output_print_def", "inputs_def", "outputs_def"]


def make_layout(ref_src):
    """sizeof/offsetof of every field of the records in the reference's own
    1DTDSE/sources/structures.h (a probe compiled against that header), with the field names
    of this package's ctypes mirrors (the reference's names), kept as record_layout.json."""
    import json
    import subprocess
    import tempfile

    from mma_gb300 import structures as S

    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "structures.h"', "int main(void){"]
    for name in LAYOUT_STRUCTS:
        cls = getattr(S, name)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(lines))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-I", ref_src, c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {k: int(v) for k, v in (l.split() for l in out if l.strip())}
    json.dump({"source": "1DTDSE/sources/structures.h", "compiler": "gcc, this machine's x86-64 ABI",
               "layout": got}, open(os.path.join(HERE, "record_layout.json"), "w"), indent=1, sort_keys=True)
    print("record_layout", len(got), "entries")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="the reference checkout (its top directory)")
    ap.add_argument("--only", choices=["tdse", "hankel", "analysis", "xuv", "radial", "ionization", "layout"],
                    default=None)
    ap.add_argument("--case", action="append", help="with --only tdse: regenerate only these TDSE fixtures")
    a = ap.parse_args()
    if a.only in (None, "tdse"):
        make_tdse(os.path.join(a.ref, "1DTDSE", "sources"), only=a.case)
    if a.only in (None, "layout"):
        make_layout(os.path.join(a.ref, "1DTDSE", "sources"))
    if a.only in (None, "hankel"):
        make_hankel(a.ref)
    if a.only in (None, "analysis"):
        make_analysis(os.path.join(a.ref, "1DTDSE", "sources"))
    if a.only in (None, "xuv"):
        make_xuv(a.ref)
    if a.only in (None, "radial"):
        make_hankel_radial(a.ref)
    if a.only in (None, "ionization"):
        make_ionization(a.ref)
