"""The oracle: CPU restatements of the reference algorithms on the 1D-TDSE -> Hankel path.

TEST INFRASTRUCTURE ONLY -- imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, and never by the product package ``mma_gb300``.

* ``tdse``   -- ctypes binding of ``_build/libmma_oracle.so`` (tdse_oracle.c), the C
  restatement of 1DTDSE/sources.  ``ref_dll_path()`` points at the reference
  DLL built unchanged from its sources (``make ref``) where those exist.
* ``hankel`` -- numpy restatement of Hankel/Hankel_transform.py.
"""
import os
import subprocess

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))


def ref_src():
    """The reference checkout's 1DTDSE/sources directory, named by the MMA_REF_SRC
    environment variable, or None when the variable is unset or names no directory."""
    src = os.environ.get("MMA_REF_SRC")
    return src if src and os.path.isdir(src) else None


def build(ref=None):
    """Compile the C restatement (always) and the reference DLL (when MMA_REF_SRC names
    the reference's sources, or when ``ref`` is True, which then requires it)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    src = ref_src()
    if ref is None:
        ref = src is not None
    if ref:
        if src is None:
            raise RuntimeError("set MMA_REF_SRC to the reference checkout's 1DTDSE/sources directory")
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref", "REF_SRC=" + src], check=True)


def ref_file(*parts):
    """Path of a file of the reference checkout (the parent of the 1DTDSE/sources directory
    named by MMA_REF_SRC), or None where the checkout is absent."""
    src = ref_src()
    if src is None:
        return None
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(src))), *parts)
    return p if os.path.exists(p) else None


def oracle_lib_path():
    return os.path.join(ORACLE_DIR, "_build", "libmma_oracle.so")


def ref_dll_path():
    """Path of the reference DLL built from its own sources, or None."""
    p = os.path.join(ORACLE_DIR, "_ref", "libsingleTDSE.so")
    return p if os.path.exists(p) else None
