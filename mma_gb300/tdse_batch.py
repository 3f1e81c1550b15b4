"""Batched TDSE on the GPU with torch tensors as device buffers.

This is the many-instance form of the reference's per-point TDSE (the MPI task
farm of 1DTDSE/sources/MPI-TDSE.c:163-178 handing (kr, kz) instances to
call1DTDSE): every instance of a batch runs in one persistent kernel launch,
instances are pulled from a device work queue, and the outputs land in device
tensors laid out [instance, ...] (instance id n = kr + kz * Nr, MPI-TDSE.c:176-178).

    grids = TDSEGrids([dict(num_r=8000, dx=0.1, trg_a=a)], dt=0.25)
    res = run_batch(grids, fields, dt_field=0.25)      # fields: [n_inst, n_f] float64 cuda
    res["sourceterm"]  # [n_inst, S]   (S = reference outputs.Nt)
    res["Fsourceterm"] # [n_inst, S//2+1] complex128

The time-grid rules are the reference's (singleTDSE.c:50-75): k1 = floor(dt_f/dt)
(+1 unless it is 1), dt' = dt_f/k1, S = k1 n_f + 2 steps.  Grids must be built
for the refined dt'.
"""
import ctypes
import math
from ctypes import POINTER, Structure, c_double, c_int, c_int64, c_size_t, c_void_p

import numpy as np
import torch

from ._lib import load

THREADS = 256
CN_SLOTS = 14  # doubles per padded site in the CN tables
GS_SLOTS = 5

PRECISIONS = {"fp64": 0, "c64": 1}
C64_SLOTS = 5  # floats per padded site in the complex64 tables


class GridRec(Structure):
    _fields_ = [("n", c_int64), ("m", c_int64), ("dx", c_double), ("trg_a", c_double), ("dt", c_double),
                ("x_int", c_double), ("Eguess", c_double), ("CV", c_double), ("max_iter", c_int64),
                ("x", c_void_p), ("gv", c_void_p), ("psi0", c_void_p), ("cn_tab", c_void_p), ("gs_tab", c_void_p),
                ("result", c_void_p), ("m32", c_int64), ("c64_tab", c_void_p)]


class InstRec(Structure):
    _fields_ = [("grid", c_int64), ("n_steps", c_int64), ("field_off", c_int64), ("n_field", c_int64),
                ("out_off", c_int64), ("psi_off", c_int64), ("snap_off", c_int64), ("snap_every", c_int64),
                ("n_snap", c_int64), ("tmin", c_double), ("gate_floor", c_double)]


class BufRec(Structure):
    _fields_ = [("fields", c_void_p), ("outputs", c_void_p), ("psi_final", c_void_p), ("snapshots", c_void_p),
                ("counter", c_void_p), ("scratch", c_void_p), ("scratch_bytes", c_size_t)]


class MMAStatusError(RuntimeError):
    pass


_STATUS = {1: "invalid argument", 2: "ground state not converged", 3: "CUDA error", 4: "cuFFT error",
           5: "too large", 6: "no CUDA device", 7: "unsupported option"}


def _check(rc, what):
    if rc != 0:
        raise MMAStatusError("%s failed: %s (status %d)" % (what, _STATUS.get(rc, "?"), rc))


def _sig():
    lib = load()
    if getattr(lib, "_mma_batch_sig", False):
        return lib
    lib.mma_tdse_build_grids.argtypes = [c_void_p, c_void_p, c_int, c_int, c_void_p]
    lib.mma_tdse_build_grids.restype = c_int
    lib.mma_tdse_propagate.argtypes = [c_void_p, c_int, c_void_p, POINTER(BufRec), c_int, c_int, c_int, c_void_p]
    lib.mma_tdse_propagate.restype = c_int
    lib.mma_tdse_scratch_bytes.argtypes = [c_int, c_int, c_int]
    lib.mma_tdse_scratch_bytes.restype = c_size_t
    lib.mma_tdse_default_ctas.argtypes = [c_int, c_int]
    lib.mma_tdse_default_ctas.restype = c_int
    lib.mma_tdse_prepare_fields.argtypes = [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]
    lib.mma_tdse_prepare_fields.restype = c_int
    lib.mma_tdse_spectra.argtypes = [c_void_p, c_int64, c_int, c_int, c_double, c_double, c_void_p, c_int64,
                                     c_void_p, c_int64, c_void_p, c_void_p]
    lib.mma_tdse_spectra.restype = c_int
    lib._mma_batch_sig = True
    return lib


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def refine(dt_field, dt_req, interp_by_dt_or_nt=0, ntinterp=1):
    """The reference's time refinement (singleTDSE.c:50-64): returns (k1, dt)."""
    if interp_by_dt_or_nt == 1:
        k1 = ntinterp + 1
    else:
        k1 = int(math.floor(dt_field / dt_req))
        if k1 != 1:
            k1 += 1
    if k1 < 1:
        raise ValueError("refinement factor must be positive")
    return k1, dt_field / k1


def n_steps(n_field, k1):
    """Propagation steps = the reference's outputs.Nt (singleTDSE.c:72,94)."""
    return k1 * n_field + 2


class TDSEGrids:
    """Device-resident grids: x, -V', ground state and solve tables of each grid.

    ``params``: list of dicts with num_r, dx, trg_a and optionally x_int (2.0),
    Eguess (-1.0), CV (1e-15), max_iter (1000).  ``dt`` is the propagation step
    (already refined).  The ground states are computed on construction.
    """

    def __init__(self, params, dt, device="cuda", stream=None, c64=False):
        lib = _sig()
        self.device = torch.device(device)
        self.dt = float(dt)
        self.params = [dict(p) for p in params]
        recs = []
        sizes = []
        for p in self.params:
            n = int(p["num_r"]) + 1
            m = (n + THREADS - 1) // THREADS
            L = m * THREADS
            sizes.append((n, m, L, n + n + 2 * n + CN_SLOTS * L + GS_SLOTS * L + 4))
        total = sum(s[3] for s in sizes)
        self.buf = torch.zeros(total, dtype=torch.float64, device=self.device)
        base = self.buf.data_ptr()
        off = 0
        self.views = []
        for p, (n, m, L, sz) in zip(self.params, sizes):
            o = off
            v = {}
            for name, cnt in (("x", n), ("gv", n), ("psi0", 2 * n), ("cn_tab", CN_SLOTS * L), ("gs_tab", GS_SLOTS * L),
                              ("result", 4)):
                v[name] = (o, cnt)
                o += cnt
            r = GridRec()
            r.n, r.m = n, m
            r.dx, r.trg_a, r.dt = float(p["dx"]), float(p["trg_a"]), self.dt
            r.x_int = float(p.get("x_int", 2.0))
            r.Eguess, r.CV = float(p.get("Eguess", -1.0)), float(p.get("CV", 1e-15))
            r.max_iter = int(p.get("max_iter", 1000))
            for name in ("x", "gv", "psi0", "cn_tab", "gs_tab", "result"):
                setattr(r, name, base + 8 * v[name][0])
            recs.append(r)
            self.views.append(v)
            off += sz
        self.n = np.array([s[0] for s in sizes])
        self.m = np.array([s[1] for s in sizes])
        self.max_m = int(self.m.max())
        self.m32 = np.array([((m + 7) // 8) * 8 for m in self.m])
        self.c64 = bool(c64)
        if self.c64:
            if self.m32.max() > 32:
                raise ValueError("the complex64 form takes grids of at most 8192 sites")
            c_sizes = C64_SLOTS * THREADS * self.m32
            self.c64_buf = torch.zeros(int(c_sizes.sum()), dtype=torch.float32, device=self.device)
            c_off = np.concatenate([[0], np.cumsum(c_sizes)])[:-1]
            for r, m32, o in zip(recs, self.m32, c_off):
                r.m32 = int(m32)
                r.c64_tab = self.c64_buf.data_ptr() + 4 * int(o)
        arr = (GridRec * len(recs))(*recs)
        self.host_recs = arr
        self.dev_recs = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(self.device)
        st = _stream_ptr(stream)
        _check(lib.mma_tdse_build_grids(ctypes.c_void_p(self.dev_recs.data_ptr()), ctypes.addressof(arr), len(recs),
                                        0, st), "mma_tdse_build_grids")
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
        if self.c64:
            lib.mma_tdse_build_c64_tables.argtypes = [c_void_p, c_void_p, c_int, c_void_p]
            lib.mma_tdse_build_c64_tables.restype = c_int
            _check(lib.mma_tdse_build_c64_tables(ctypes.c_void_p(self.dev_recs.data_ptr()), ctypes.addressof(arr),
                                                 len(recs), st), "mma_tdse_build_c64_tables")
            torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
        res = np.stack([self._view(g, "result").cpu().numpy() for g in range(len(recs))])
        self.Einit = res[:, 0].copy()
        self.iterations = res[:, 1].astype(int)
        self.status = res[:, 2].astype(int)
        if np.any(self.status != 0):
            bad = np.nonzero(self.status)[0]
            raise MMAStatusError("ground state not converged for grids %s" % bad.tolist())

    def _view(self, g, name):
        o, c = self.views[g][name]
        return self.buf[o:o + c]

    def x(self, g=0):
        return self._view(g, "x")

    def psi0(self, g=0):
        v = self._view(g, "psi0")
        return torch.view_as_complex(v.view(-1, 2))

    def __len__(self):
        return len(self.params)


class BatchResult(dict):
    """Packed outputs of a batch; ``series(i)`` gives instance i's six series."""

    def series(self, i):
        o, S = self["out_off"][i], self["S"][i]
        blk = self["outputs"][o:o + 6 * (S + 1)].view(6, S + 1)
        return {k: blk[s, :S] for s, k in enumerate(("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval"))}


def run_batch(grids, fields, dt_field, grid_ids=None, dt_req=None, tmin=0.0, spectra=True, psi_final=False,
              snap_every=0, precision="fp64", grid_ctas=0, stream=None, tmax=None, _events=None):
    """Propagate a batch of instances.

    fields: float64 cuda tensor [n_inst, n_f] (uniform) or a list of 1-D tensors
    (uneven lengths).  grid_ids: per-instance grid index (default all 0).
    Returns a BatchResult with packed ``outputs`` plus, for uniform batches, views
    ``sourceterm``, ``PopTot``, ``PopInt``, ``expval``, ``Efield``, ``tgrid``
    [n_inst, S] and spectra ``Fsourceterm`` [n_inst, S//2+1] (complex128),
    ``FsourcetermM2``, ``omegagrid``.
    """
    lib = _sig()
    if precision not in PRECISIONS:
        raise ValueError("precision must be one of %s" % list(PRECISIONS))
    dev = grids.device
    uniform = torch.is_tensor(fields) and fields.dim() == 2
    rows = [fields[i] for i in range(fields.shape[0])] if uniform else list(fields)
    n_inst = len(rows)
    if n_inst == 0:
        raise ValueError("empty batch")
    k1, dt = refine(dt_field, dt_req if dt_req is not None else grids.dt)
    if abs(dt - grids.dt) > 1e-12 * grids.dt:
        raise ValueError("grids were built for dt=%g but this batch refines to dt=%g" % (grids.dt, dt))
    gid = np.zeros(n_inst, dtype=np.int64) if grid_ids is None else np.asarray(grid_ids, dtype=np.int64)
    if gid.shape != (n_inst,) or gid.min() < 0 or gid.max() >= len(grids):
        raise ValueError("grid_ids must index the grids")
    nf = np.array([int(r.numel()) for r in rows], dtype=np.int64)
    if nf.min() < 2:
        raise ValueError("every field needs at least 2 samples")
    st = _stream_ptr(stream)
    S = n_steps(nf, k1)
    # refined fields, grouped by raw length for batched interpolation
    fld_off = np.concatenate([[0], np.cumsum(k1 * nf)])[:-1]
    fld = torch.empty(int((k1 * nf).sum()), dtype=torch.float64, device=dev)
    gate_floor = np.zeros(n_inst)
    for L in np.unique(nf):
        idx = np.nonzero(nf == L)[0]
        raw = torch.stack([rows[i].to(device=dev, dtype=torch.float64) for i in idx]) if not uniform else \
            fields[torch.as_tensor(idx, device=dev)].to(torch.float64).contiguous()
        if not torch.isfinite(raw).all():
            raise ValueError("field has non-finite samples")
        out = torch.empty(len(idx), k1 * int(L), dtype=torch.float64, device=dev)
        _check(lib.mma_tdse_prepare_fields(raw.data_ptr(), len(idx), int(L), k1, out.data_ptr(), st),
               "mma_tdse_prepare_fields")
        if k1 > 1:
            gate_floor[idx] = 1e-13 * raw.abs().amax(dim=1).cpu().numpy()
        for j, i in enumerate(idx):
            fld[fld_off[i]:fld_off[i] + k1 * L].copy_(out[j])
    out_off = np.concatenate([[0], np.cumsum(6 * (S + 1))])[:-1]
    outputs = torch.zeros(int((6 * (S + 1)).sum()), dtype=torch.float64, device=dev)
    psi_off = np.full(n_inst, -1, dtype=np.int64)
    psi_buf = None
    if psi_final:
        sizes = 2 * grids.n[gid]
        psi_off = np.concatenate([[0], np.cumsum(sizes)])[:-1]
        psi_buf = torch.zeros(int(sizes.sum()), dtype=torch.float64, device=dev)
    snap_off = np.full(n_inst, -1, dtype=np.int64)
    n_snap = np.zeros(n_inst, dtype=np.int64)
    snap_buf = None
    if snap_every:
        n_snap = S // snap_every
        sizes = n_snap * 2 * grids.n[gid]
        snap_off = np.concatenate([[0], np.cumsum(sizes)])[:-1]
        snap_buf = torch.zeros(int(sizes.sum()), dtype=torch.float64, device=dev)
    insts = (InstRec * n_inst)()
    for i in range(n_inst):
        r = insts[i]
        r.grid, r.n_steps, r.field_off, r.n_field = int(gid[i]), int(S[i]), int(fld_off[i]), int(k1 * nf[i])
        r.out_off, r.psi_off, r.snap_off = int(out_off[i]), int(psi_off[i]), int(snap_off[i])
        r.snap_every, r.n_snap = max(int(snap_every), 1), int(n_snap[i]) if snap_every else 0
        r.tmin, r.gate_floor = float(tmin), float(gate_floor[i])
    d_insts = torch.frombuffer(bytearray(bytes(insts)), dtype=torch.uint8).to(dev)
    max_m = int(grids.m[np.unique(gid)].max())
    prec = PRECISIONS[precision]
    if prec == 1:
        if not grids.c64:
            raise ValueError("build the grids with c64=True for the complex64 form")
        m32s = np.unique(grids.m32[np.unique(gid)])
        if len(m32s) != 1:
            raise ValueError("one complex64 launch needs grids of one m32; split the batch by grids.m32")
        max_m = int(m32s[0])
    ctas = grid_ctas or lib.mma_tdse_default_ctas(max_m, prec)
    ctas = min(ctas, n_inst)
    sbytes = lib.mma_tdse_scratch_bytes(max_m, ctas, prec)
    scratch = torch.empty(max(int(sbytes), 8), dtype=torch.uint8, device=dev)
    counter = torch.zeros(1, dtype=torch.int32, device=dev)
    B = BufRec(fld.data_ptr(), outputs.data_ptr(), psi_buf.data_ptr() if psi_buf is not None else None,
               snap_buf.data_ptr() if snap_buf is not None else None, counter.data_ptr(), scratch.data_ptr(),
               int(sbytes))
    if _events is not None:  # timing hook: events around the propagation launch only
        _events[0].record(stream if stream is not None else torch.cuda.current_stream())
    _check(lib.mma_tdse_propagate(d_insts.data_ptr(), n_inst, grids.dev_recs.data_ptr(), ctypes.byref(B), max_m, ctas,
                                  prec, st), "mma_tdse_propagate")
    if _events is not None:
        _events[1].record(stream if stream is not None else torch.cuda.current_stream())
    res = BatchResult(outputs=outputs, out_off=out_off, S=S, k1=k1, dt=dt, n_field=nf, psi_off=psi_off,
                      psi_final=psi_buf, snapshots=snap_buf, snap_off=snap_off, n_snap=n_snap, grid_ids=gid,
                      ctas=ctas, _keep=(d_insts, scratch, counter, fld))
    if uniform and len(np.unique(S)) == 1:
        s = int(S[0])
        blk = outputs.view(n_inst, 6, s + 1)
        for j, k in enumerate(("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval")):
            res[k] = blk[:, j, :s]
        if spectra:
            nc = s // 2 + 1
            if tmax is None:  # the reference's tgrid[Nf-1] - tgrid[0] (singleTDSE.c:50)
                tmax = (int(nf[0]) - 1) * dt_field
            fs = torch.empty(n_inst, 2 * nc, dtype=torch.float64, device=dev)
            fm = torch.empty(n_inst, nc, dtype=torch.float64, device=dev)
            om = torch.empty(nc, dtype=torch.float64, device=dev)
            _check(lib.mma_tdse_spectra(outputs.data_ptr() + 8 * 2 * (s + 1), 6 * (s + 1), n_inst, s, dt, tmax,
                                        fs.data_ptr(), 2 * nc, fm.data_ptr(), nc, om.data_ptr(), st),
                   "mma_tdse_spectra")
            res["Fsourceterm"] = torch.view_as_complex(fs.view(n_inst, nc, 2))
            res["FsourcetermM2"] = fm
            res["omegagrid"] = om
    return res
