"""The C-ABI boundary without a GPU: the library loads, exports every entry point
declared in include/*.h, its records have the reference's byte layout, and the
legacy calls report (rather than crash on) a missing device or bad arguments."""
import ctypes
import glob
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = "\n".join(l for l in src.split("\n") if not l.strip().startswith("#"))
        src = src.replace('extern "C" {', "")
        depth = 0
        stmt = ""
        for ch in src:
            if ch == "{":
                depth += 1
            elif ch == "}":
                depth = max(depth - 1, 0)
                stmt = ""
                continue
            if depth:
                continue
            if ch == ";":
                s = " ".join(stmt.split())
                stmt = ""
                if s.startswith("typedef") or s.startswith("#") or "(" not in s:
                    continue
                m = re.match(r"^(?:extern\s+\"C\"\s+)?[\w\s\*]+?\**\s*(\w+)\s*\(", s)
                if m:
                    names.append(m.group(1))
            else:
                stmt += ch
    return sorted(set(names))


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "call1DTDSE" in names and "mma_tdse_propagate" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    from mma_gb300 import load

    lib = load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


STRUCTS = ["Efield_var", "trg_def", "analy_def", "output_print_def", "inputs_def", "outputs_def"]


def test_record_layout_matches_header():
    """Compile a probe against include/mma_tdse.h and compare sizeof/offsetof with the
    ctypes mirrors (which follow 1DTDSE/sources/structures.h)."""
    from mma_gb300 import structures as S

    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mma_tdse.h"', "int main(void){"]
    for name in STRUCTS:
        cls = getattr(S, name)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(lines))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(l.split() for l in out if l.strip())
    for name in STRUCTS:
        cls = getattr(S, name)
        assert int(got[name]) == ctypes.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(got[name + "." + f]) == getattr(cls, f).offset, (name, f)


def test_batched_records_are_8_byte_fields():
    src = open(os.path.join(ROOT, "include", "mma_tdse.h")).read()
    for rec in ("mma_tdse_grid", "mma_tdse_instance"):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (rec, rec), src, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        for decl in body.split(";"):
            decl = decl.strip()
            if decl:  # pointers, int64_t and double only: 8-byte fields, no padding
                assert "*" in decl or decl.split()[0] in ("int64_t", "double"), decl


def test_legacy_calls_report_errors_without_crashing():
    """Bad arguments (or, on a machine without a GPU, the missing device) come back as a
    status, never as exit() or a crash; no kernel runs on these paths."""
    from mma_gb300.structures import inputs_def, outputs_def
    from mma_gb300.tdse import MMAError, TDSE_DLL

    dll = TDSE_DLL()
    inp = inputs_def()
    inp.init_default_inputs(num_r=1)  # too small: rejected before any device work
    with pytest.raises(MMAError):
        dll.init_GS(inp)
    out = outputs_def()
    with pytest.raises(MMAError):
        dll.call1DTDSE(inp, out)  # no field, no ground state
    t = np.linspace(0, 10, 41)
    E = np.zeros_like(t)
    E[3] = np.nan
    inp2 = inputs_def()
    inp2.init_default_inputs(num_r=100, dx=0.4)
    from mma_gb300.tdse import init_time_and_field

    init_time_and_field(dll, inp2, t, E)
    import ctypes as C

    n = 101
    xs = (C.c_double * n)(*np.linspace(-20, 20, n))
    ps = (C.c_double * (2 * n))()
    inp2.x = C.cast(xs, C.POINTER(C.c_double))
    inp2.psi0 = C.cast(ps, C.POINTER(C.c_double))
    with pytest.raises(MMAError, match="non-finite"):
        dll.call1DTDSE(inp2, out)
    inp2.gauge = 1
    E[3] = 0.0


def test_c64_shapes():
    """Kernel shapes of the complex64 form (no GPU call)."""
    from mma_gb300.autotune import candidate_shapes

    assert candidate_shapes(8001) == [(256, 32), (512, 16), (1024, 8)]
    assert candidate_shapes(12001) == [(256, 48)]
    assert candidate_shapes(601) == [(256, 8), (512, 8), (1024, 8)]


def test_batched_record_layouts_match_mirrors():
    """sizeof/offsetof of the batched and far-field records against their ctypes mirrors."""
    from mma_gb300.hankel import FastPlan, HankelProblem
    from mma_gb300.tdse_batch import BufRec, GridRec, InstRec

    pairs = [("mma_tdse_grid", GridRec), ("mma_tdse_instance", InstRec), ("mma_tdse_buffers", BufRec),
             ("mma_hankel_problem", HankelProblem), ("mma_hankel_fast_plan_t", FastPlan)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mma_tdse.h"', '#include "mma_hankel.h"',
             "int main(void){"]
    for cname, cls in pairs:
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(lines))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(l.split() for l in out if l.strip())
    for cname, cls in pairs:
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(got[cname + "." + f]) == getattr(cls, f).offset, (cname, f)


def _probe_layout(header_dir, header, names):
    from mma_gb300 import structures as S

    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "%s"' % header, "int main(void){"]
    for name in names:
        cls = getattr(S, name)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(lines))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-I", header_dir, c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    return {k: int(v) for k, v in (l.split() for l in out if l.strip())}


def test_record_layout_matches_reference_header():
    """The records' sizeof/offsetof as the reference's own 1DTDSE/sources/structures.h lays them
    out (tests/golden/record_layout.json, from a probe compiled against that header by
    tests/golden/make_golden.py --only layout) equal this repository's header and ctypes mirrors;
    where the reference checkout is named by MMA_REF_SRC the probe is also rebuilt against it."""
    import json

    from mma_gb300 import structures as S

    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "record_layout.json")))["layout"]
    ours = _probe_layout(os.path.join(ROOT, "include"), "mma_tdse.h", STRUCTS)
    assert ours == ref
    for name in STRUCTS:
        cls = getattr(S, name)
        assert ref[name] == ctypes.sizeof(cls), name
        for f, _ in cls._fields_:
            assert ref[name + "." + f] == getattr(cls, f).offset, (name, f)
    import oracle

    src = oracle.ref_src()
    if src is not None:
        assert _probe_layout(src, "structures.h", STRUCTS) == ref


def test_reference_host_class_binds_this_library():
    """The reference's own, unmodified host class (1DTDSE/PythonTDSE.py and PythonCTDSE/*.py,
    imported from the checkout named by MMA_REF_SRC; h5py, matplotlib and MMA_administration,
    which this path does not use, stubbed) loads libmma_gb300.so: every symbol it binds
    resolves, and its call sequence -- default inputs, field, ground state, propagation --
    returns without exiting; with no GPU the library records MMA_ERR_NO_DEVICE (6) for the ground
    state, and the propagation without a ground state is refused with a status."""
    import importlib
    import sys
    import types

    import oracle

    top = oracle.ref_file("1DTDSE")
    if top is None:
        pytest.skip("the reference checkout is not named here (MMA_REF_SRC)")
    import torch

    if torch.cuda.is_available():
        pytest.skip("checks the no-device path; the GPU tests cover the computation")
    from mma_gb300._lib import lib_path

    saved = dict(sys.modules)
    saved_path = list(sys.path)
    try:
        for name in ("h5py", "matplotlib", "matplotlib.pyplot", "matplotlib.colors", "MMA_administration"):
            sys.modules[name] = types.ModuleType(name)
        sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
        sys.modules["matplotlib"].colors = sys.modules["matplotlib.colors"]
        sys.modules["matplotlib.colors"].LogNorm = sys.modules["matplotlib.colors"].Normalize = object
        for name in [m for m in sys.modules if m == "PythonTDSE" or m.startswith("PythonCTDSE")]:
            del sys.modules[name]
        sys.path.insert(0, top)
        try:
            PT = importlib.import_module("PythonTDSE")
        except ImportError as e:
            pytest.skip("the reference host class needs %s here" % e.name)
        dll = PT.TDSE_DLL(lib_path())
        for sym in ("Initialise_grid_and_ground_state", "call1DTDSE", "window_analysis", "GaborTransform",
                    "free_mtrx", "free_arr", "outputs_destructor", "inputs_destructor", "set_time_and_field",
                    "Set_all_prints"):
            assert hasattr(dll.DLL, sym), sym
        inp = PT.inputs_def()
        inp.init_default_inputs(num_r=600, dx=0.4)
        t = np.linspace(0.0, 50.0, 201)
        inp.init_time_and_field(dll, E=0.05 * np.sin(0.057 * t), t=t)
        out = PT.outputs_def()
        dll.DLL.mma_last_error.restype = ctypes.c_int
        dll.init_GS(inp)
        assert dll.DLL.mma_last_error() == 6  # no device: reported, not exit()
        dll.call1DTDSE(inp, out)
        assert dll.DLL.mma_last_error() in (1, 6)  # no ground state (argument check) or no device
    finally:
        sys.modules.clear()
        sys.modules.update(saved)
        sys.path[:] = saved_path
