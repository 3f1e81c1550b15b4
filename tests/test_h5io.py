"""HDF5 archives: the package's own reader/writer (mma_gb300.h5io), the records' save/load methods,
the archive drivers (mma_gb300.archive), and the reference's stored regression results.

The reference keeps one regression archive, 1DTDSE/ionization.h5, written by its
``save_to_hdf5`` after the run in 1DTDSE/tests.py:13-39 (trg_a = 1, dx = 0.4, num_r = 8000,
dt = 0.25, E0 = 0.14, omega = 0.07, 4 cycles, snapshots every 10 a.u.) and read back by its tests
(tests.py:50-88), which compare with np.allclose.  tests/golden/ionization_h5.npz holds its
datasets as stored (float32 / int32; the snapshots every 7th), read with mma_gb300.h5io
(tests/golden/make_golden.py).  The archive stores float32, so the bound for values computed
here in FP64 is float32 rounding: relative error <= 1.2e-7 of the largest value, besides the
reference's own np.allclose.
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
F32_REL = 1.2e-7


def _fix():
    return np.load(os.path.join(GOLDEN, "ionization_h5.npz"))


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


def _tests_py_case():
    """The field of 1DTDSE/tests.py:14-33."""
    E0, omega, n_cycles, dt = 0.14, 0.07, 4, 0.25
    T_max = n_cycles * 2 * np.pi / omega
    t = np.linspace(0, T_max, int(T_max / dt) + 1)
    return t, E0 * np.sin(np.pi * t / T_max) ** 2 * np.cos(omega * t)


def _write_fixture_archive(path, g):
    """The fixture written back as an archive in the reference's layout."""
    from mma_gb300 import h5io

    with h5io.File(path, "w") as f:
        for k in g.files:
            if "__" in k:
                grp, name = k.split("__", 1)
                f.create_dataset(grp + "/" + name, data=g[k])


def _check_against_archive(g, x, psi0, Einit, o, snapshots):
    """Results of the tests.py run against the archive: the reference's np.allclose and float32
    rounding of the largest value."""
    assert np.float32(Einit) == g["TDSE_inputs__Einit"]
    assert np.array_equal(np.float32(x), g["TDSE_inputs__x_grid"])
    assert np.array_equal(np.float32(np.stack([psi0.real, psi0.imag], 1)), g["TDSE_inputs__psi0"])
    assert int(g["TDSE_outputs__Nt"]) == len(o["sourceterm"]) and int(g["TDSE_outputs__Nomega"]) == len(o["omegagrid"])
    for k in ("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval", "omegagrid"):
        ref = g["TDSE_outputs__" + k]
        assert np.allclose(ref, o[k]), k
        assert _rel(o[k], ref) < F32_REL, k
    for k in ("Fsourceterm", "FEfield"):
        v = np.stack([o[k].real, o[k].imag], 1)
        assert np.allclose(g["TDSE_outputs__" + k], v), k
        assert _rel(v, g["TDSE_outputs__" + k]) < F32_REL, k
    s = snapshots[g["snapshot_index"]]
    for part, ref in ((s.real, g["TDSE_outputs__psi_re"]), (s.imag, g["TDSE_outputs__psi_im"])):
        assert np.allclose(ref, part) and _rel(part, ref) < F32_REL


def test_reader_reads_reference_archive():
    """The reference's own archive (written by libhdf5) read with mma_gb300.h5io."""
    import oracle
    from mma_gb300 import h5io

    path = oracle.ref_file("1DTDSE", "ionization.h5")
    if path is None:
        pytest.skip("reference checkout not present")
    g = _fix()
    f = h5io.File(path)
    assert sorted(f.keys()) == ["TDSE_inputs", "TDSE_outputs"]
    n = 0
    for grp in ("TDSE_inputs", "TDSE_outputs"):
        for k in f[grp].keys():
            v = f[grp + "/" + k][()]
            if k in ("psi_re", "psi_im"):
                v = v[g["snapshot_index"]]
            ref = g[grp + "__" + k]
            assert np.asarray(v).dtype == ref.dtype and np.array_equal(v, ref), k
            n += 1
    assert n == len(g.files) - 1


def test_oracle_reproduces_reference_archive(oracle_built):
    import oracle.tdse as ot

    g = _fix()
    t, E = _tests_py_case()
    assert np.array_equal(np.float32(t), g["TDSE_inputs__tgrid"])
    x, psi0, Einit, _ = ot.ground_state(8000, 0.4, 1.0, -1.0, 1e-15)
    o = ot.propagate(x, psi0, t, E, 0.4, 1.0, writewft=1, tprint=10.0)
    _check_against_archive(g, x, psi0, Einit, o, o["snapshots"])


def test_writer_round_trip(tmp_path):
    from mma_gb300 import h5io

    rng = np.random.default_rng(0)
    data = {
        "a/f8": rng.standard_normal((3, 4, 2)),
        "a/f4": rng.standard_normal(7).astype(np.float32),
        "a/i4": np.arange(5, dtype=np.int32),
        "a/i8": np.int64(-3),
        "a/u1": np.arange(3, dtype=np.uint8),
        "a/b/c/deep": np.array([1.5]),
        "s": np.bytes_("text"),
        "empty": np.zeros(0),
    }
    for i in range(70):  # more members than one symbol node holds
        data["many/m%02d" % (69 - i)] = np.full(i + 1, float(i))
    p = str(tmp_path / "t.h5")
    with h5io.File(p, "w") as f:
        for k, v in data.items():
            f.create_dataset(k, data=v)
        f["a/f8"].attrs["units"] = np.bytes_("[a.u.]")
        f["a"].attrs["n"] = np.int32(4)
    r = h5io.File(p)
    for k, v in data.items():
        got = r[k][()]
        assert np.shape(got) == np.shape(v) and np.asarray(got).dtype == np.asarray(v).dtype, k
        assert np.array_equal(got, v), k
    assert r["a/f8"].attrs["units"] == b"[a.u.]" and int(r["a"].attrs["n"]) == 4
    assert sorted(r["many"].keys()) == sorted("m%02d" % i for i in range(70))
    assert "a/b/c" in r and "a/x" not in r
    # the superblock of a new file at libhdf5's default format version: signature, versions 0,
    # 8-byte offsets and lengths, group leaf K 4 and internal K 16 (the reference archive's bytes)
    with open(p, "rb") as fh:
        assert fh.read(24) == bytes.fromhex("894844460d0a1a0a00000000000808000400100000000000")


def test_chunked_and_filtered_round_trip(tmp_path):
    """Chunked datasets (B-tree v1 chunk index, as CUPRAD's unlimited datasets are stored), edge
    chunks, a multi-level index and the deflate and shuffle filters."""
    from mma_gb300 import h5io

    rng = np.random.default_rng(2)
    data = {"a": (rng.standard_normal((37, 50, 3)), dict(chunks=(8, 16, 3), compression="gzip", shuffle=True)),
            "b": (np.arange(1000, dtype=np.int32).reshape(10, 100), dict(chunks=(3, 7))),
            "c": (rng.standard_normal(5000).astype(np.float32), dict(chunks=(10,), compression="gzip",
                                                                      compression_opts=9)),
            "d": (rng.standard_normal((4, 6)), dict(compression="gzip"))}
    p = str(tmp_path / "c.h5")
    with h5io.File(p, "w") as f:
        for k, (v, kw) in data.items():
            f.create_dataset(k, data=v, **kw)
    r = h5io.File(p)
    for k, (v, _) in data.items():
        assert r[k].dtype == v.dtype and np.array_equal(r[k][()], v), k
    with pytest.raises(ValueError):
        h5io.File(str(tmp_path / "x.h5"), "w").create_dataset("x", data=np.zeros((2, 2)), chunks=(2,))


def test_append_keeps_existing(tmp_path):
    from mma_gb300 import h5io

    p = str(tmp_path / "a.h5")
    with h5io.File(p, "w") as f:
        f.create_dataset("g/x", data=np.arange(4.0)).attrs["units"] = np.bytes_("[m]")
    with h5io.File(p, "a") as f:
        f.require_group("g").create_dataset("y", data=np.int32(7))
        with pytest.raises(ValueError):
            f.create_dataset("g/x", data=np.zeros(1))
    r = h5io.File(p)
    assert np.array_equal(r["g/x"][()], np.arange(4.0)) and r["g/x"].attrs["units"] == b"[m]"
    assert int(r["g/y"][()]) == 7


def test_records_load_and_save(tmp_path):
    """inputs_def / outputs_def load_from_hdf5 and save_to_hdf5 in the reference's layout
    (PythonCTDSE/structures.py:133-166, 301-340, 454-545): an archive round trip is exact."""
    from mma_gb300 import h5io
    from mma_gb300.structures import inputs_def, outputs_def

    g = _fix()
    src = str(tmp_path / "src.h5")
    _write_fixture_archive(src, g)
    inp, out = inputs_def(), outputs_def()
    inp.load_from_hdf5(src)
    out.load_from_hdf5(src)
    assert inp.num_r == 8000 and abs(inp.dx - 0.4) < 1e-7 and inp.analy.writewft == 1
    assert np.array_equal(inp.get_xgrid(), g["TDSE_inputs__x_grid"])
    assert np.array_equal(out.get_sourceterm(), g["TDSE_outputs__sourceterm"])
    assert np.array_equal(out.get_Fsourceterm(), g["TDSE_outputs__Fsourceterm"][:, 0] + 1j * g["TDSE_outputs__Fsourceterm"][:, 1])
    wf = out.get_wavefunction(inp, grids=False)
    assert np.array_equal(wf.real, g["TDSE_outputs__psi_re"])
    tg, x, wf2 = out.get_wavefunction(inp)
    assert len(tg) == wf.shape[0] and np.array_equal(x, inp.get_xgrid())
    dst = str(tmp_path / "dst.h5")
    inp.save_to_hdf5(dst)
    out.save_to_hdf5(dst, inputs=inp)
    r = h5io.File(dst)
    for k in g.files:
        if "__" in k:
            grp, name = k.split("__", 1)
            if name == "num_t":
                continue  # not a loaded input
            v = r[grp + "/" + name][()]
            assert np.asarray(v).dtype == g[k].dtype and np.array_equal(v, g[k]), k


def _cuprad_archive(path, n_z=4, n_t=600, n_r=5):
    """A synthetic macroscopic archive: CUPRAD/outputs/{output_field [z, t, r] (V/m), tgrid (s),
    rgrid, zgrid (m)} and CTDSE/inputs coarsening parameters."""
    from mma_gb300 import h5io
    from mma_gb300.archive import EFIELDau, TIMEau

    t_au = np.arange(n_t) * 0.25
    r = np.linspace(0, 80e-6, n_r)
    z = np.linspace(-1e-3, 1e-3, n_z)
    T = t_au[-1]
    env = np.sin(np.pi * t_au / T) ** 2 * np.cos(0.057 * t_au)
    amp = 0.06 * np.exp(-(r / 60e-6) ** 2)[None, :] * (1.0 - 0.05 * np.arange(n_z))[:, None]
    E = amp[:, None, :] * env[None, :, None] * EFIELDau
    with h5io.File(path, "w") as f:
        f.create_dataset("CUPRAD/outputs/output_field", data=E)
        f.create_dataset("CUPRAD/outputs/tgrid", data=t_au * TIMEau)
        f.create_dataset("CUPRAD/outputs/rgrid", data=r)
        f.create_dataset("CUPRAD/outputs/zgrid", data=z)
        for k, v in (("kz_step", 1), ("kr_step", 2), ("Nz_max", n_z), ("Nr_max", n_r)):
            f.create_dataset("CTDSE/inputs/" + k, data=np.int32(v))
    return t_au, E / EFIELDau, r, z


def test_read_cuprad_fields(tmp_path):
    from mma_gb300.archive import read_cuprad_fields

    p = str(tmp_path / "in.h5")
    t_au, E_au, r, z = _cuprad_archive(p)
    d = read_cuprad_fields(p)
    assert np.allclose(d["tgrid"], t_au, rtol=1e-14, atol=1e-14)
    assert d["n_z"] == 4 and d["n_r"] == 2  # Nr_max // kr_step = 5 // 2 (tools_algorithmic.c:56)
    assert np.array_equal(d["rgrid_coarse"], r[[0, 2]]) and np.array_equal(d["zgrid_coarse"], z)
    for kz in range(4):
        for kr in range(2):  # instance n = kr + kz Nr
            assert np.allclose(d["fields"][kr + kz * 2], E_au[kz, :, 2 * kr], rtol=1e-14, atol=1e-20)
    with pytest.raises(ValueError):
        read_cuprad_fields(p, Nr_max=6)


def test_ctdse_and_dynamic_source_layout(tmp_path):
    """write_ctdse_outputs in the merged layout (merge.py:71-108) and the far-field provider
    reading it back ('dynamic', Hankel_transform.py:71-77), on a synthetic result."""
    from mma_gb300 import h5io
    from mma_gb300.archive import write_ctdse_outputs
    from mma_gb300.hankel import FSources_provider

    rng = np.random.default_rng(1)
    n_z, n_r, S, No = 3, 4, 16, 9
    n = n_z * n_r
    res = {k: rng.standard_normal((n, S)) for k in ("Efield", "sourceterm", "PopInt", "expval")}
    res["tgrid"] = np.tile(np.arange(S) * 0.25, (n, 1))
    res["omegagrid"] = np.arange(No) * 0.1
    res["Fsourceterm"] = rng.standard_normal((n, No)) + 1j * rng.standard_normal((n, No))
    p = str(tmp_path / "o.h5")
    rc, zc = np.linspace(0, 1e-4, n_r), np.linspace(-1e-3, 1e-3, n_z)
    write_ctdse_outputs(p, res, n_r, n_z, rc, zc)
    f = h5io.File(p)
    g = f["CTDSE/outputs"]
    assert g["SourceTerm"].shape == (n_z, n_r, S) and g["FSourceTerm"].shape == (n_z, n_r, No, 2)
    assert g["SourceTerm"].attrs["units"] == b"[a.u.]" and g["PopInt"].attrs["units"] == b"[-]"
    kz, kr = 2, 1
    assert np.array_equal(g["SourceTerm"][()][kz, kr], res["sourceterm"][kr + kz * n_r])
    assert np.array_equal(g["FSourceTermM2"][()][kz, kr], np.abs(res["Fsourceterm"][kr + kz * n_r]) ** 2)
    ogrid = np.linspace(1e15, 2e15, No)
    prov = FSources_provider(zc, rc, ogrid, data_source="dynamic", h5_handle=f, h5_path="CTDSE/outputs/FSourceTerm",
                             ko_min=2, ko_max=8, ko_step=2, device="cpu")
    planes = list(prov.Fsource_plane)
    assert len(planes) == n_z - 1  # the last plane is dropped (Hankel_transform.py:62)
    F = res["Fsourceterm"].reshape(n_z, n_r, No)
    for k, pl in enumerate(planes):
        assert np.array_equal(pl.numpy(), F[k, :, 2:8:2].T)


@pytest.mark.gpu
def test_library_reproduces_reference_archive(gpu_lib, tmp_path):
    """1DTDSE/tests.py run through this library's legacy symbols, compared with the reference's
    archive loaded through outputs_def.load_from_hdf5, as the reference's test_outputs does."""
    from mma_gb300.structures import inputs_def, outputs_def
    from mma_gb300.tdse import TDSE_DLL

    g = _fix()
    dll = TDSE_DLL()
    inp = inputs_def()
    inp.init_default_inputs(trg_a=1.0, CV=1e-15, num_r=8000)
    t, E = _tests_py_case()
    inp.init_time_and_field(dll, t=t, E=E)
    inp.analy.writewft = 1
    inp.analy.tprint = 10.0
    dll.init_GS(inp)
    out = outputs_def()
    dll.call1DTDSE(inp, out)
    src = str(tmp_path / "ionization.h5")
    _write_fixture_archive(src, g)
    ref = outputs_def()
    ref.load_from_hdf5(src)
    assert ref.Nt == out.Nt and ref.Nomega == out.Nomega
    o = {k: getattr(out, "get_" + k)() for k in ("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval",
                                                 "omegagrid", "Fsourceterm", "FEfield")}
    _check_against_archive(g, inp.get_xgrid(), inp.get_GS(), inp.Einit, o, out.get_wavefunction(inp, grids=False))


@pytest.mark.gpu
def test_archive_to_archive_pipeline(gpu_lib, oracle_built, tmp_path):
    """Macroscopic archive -> TDSE batch -> CTDSE/outputs (merged layout) -> far field from the
    archive ('dynamic' source) -> Hankel/outputs, against the oracle composition in FP64
    (relative error <= 1e-8 of the largest far-field value)."""
    import torch

    import oracle.hankel as oh
    import oracle.tdse as ot
    from mma_gb300 import h5io
    from mma_gb300 import hankel as H
    from mma_gb300.archive import read_cuprad_fields, write_ctdse_outputs, write_hankel_outputs
    from mma_gb300.pipeline import OMEGA_AU2SI, harmonic_window
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    p = str(tmp_path / "run.h5")
    _cuprad_archive(p)
    d = read_cuprad_fields(p)
    num_r, dx, a = 600, 0.4, 1.0
    dtf = float(d["tgrid"][1] - d["tgrid"][0])
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=a)], dt=dtf)
    res = run_batch(grids, torch.tensor(d["fields"], device="cuda"), dtf, precision="fp64",
                    tmax=float(d["tgrid"][-1] - d["tgrid"][0]))
    write_ctdse_outputs(p, res, d["n_r"], d["n_z"], d["rgrid_coarse"], d["zgrid_coarse"], grids=grids)
    n_xuv = complex(1 - 1e-5, 1e-7)
    H.XUV_index.set_constant_index(n_xuv)
    rho = np.linspace(0.0, 2e-3, 12)
    f = h5io.File(p)
    og_au = f["CTDSE/outputs/omegagrid"][()]
    ko_min, ko_max = harmonic_window(og_au, 0.057, (3.0, 15.0))
    target = H.FSources_provider(f["CTDSE/outputs/zgrid_coarse"][()], f["CTDSE/outputs/rgrid_coarse"][()],
                                 OMEGA_AU2SI * og_au, data_source="dynamic", h5_handle=f,
                                 h5_path="CTDSE/outputs/FSourceTerm", ko_min=ko_min, ko_max=ko_max)
    far = H.Hankel_long(target, 1.0, rho, preset_gas="Ar", form="plain")
    write_hankel_outputs(p, far)
    r = h5io.File(p)
    FF = r["Hankel/outputs/FF_integrated"][()]
    assert FF.shape == (len(rho), ko_max - ko_min, 2)
    assert int(r["CTDSE/outputs/SourceTerm"].shape[0]) == d["n_z"]
    # oracle composition
    x, psi0, _, _ = ot.ground_state(num_r, dx, a, -1.0, 1e-15)
    spec = [ot.propagate(x, psi0, d["tgrid"], d["fields"][n], dx, a)["Fsourceterm"] for n in range(len(d["fields"]))]
    F = np.stack(spec).reshape(d["n_z"], d["n_r"], -1)
    S = F[:, :, ko_min:ko_max].transpose(0, 2, 1)
    og_si = OMEGA_AU2SI * og_au[ko_min:ko_max]
    disp, absorb = oh.constant_index_factors(og_si, n_xuv)
    ref = oh.hankel_long(d["zgrid_coarse"], d["rgrid_coarse"], og_si, S, 1.0, rho, disp=disp, absorb=absorb)
    got = FF[..., 0] + 1j * FF[..., 1]
    assert np.abs(got - ref["FF_integrated"]).max() < 1e-8 * np.abs(ref["FF_integrated"]).max()
