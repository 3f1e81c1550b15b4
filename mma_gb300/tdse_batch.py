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

PRECISIONS = {"fp64": 0, "c64": 1, "df64": 2}
C64_SLOTS = 5  # floats per padded site in the complex64 tables


class GridRec(Structure):
    _fields_ = [("n", c_int64), ("m", c_int64), ("dx", c_double), ("trg_a", c_double), ("dt", c_double),
                ("x_int", c_double), ("Eguess", c_double), ("CV", c_double), ("max_iter", c_int64),
                ("x", c_void_p), ("gv", c_void_p), ("psi0", c_void_p), ("cn_tab", c_void_p), ("gs_tab", c_void_p),
                ("result", c_void_p), ("m32", c_int64), ("c64_tab", c_void_p), ("adj_tab", c_void_p),
                ("c64_threads", c_int64), ("df_tab", c_void_p)]


class InstRec(Structure):
    _fields_ = [("grid", c_int64), ("n_steps", c_int64), ("field_off", c_int64), ("n_field", c_int64),
                ("out_off", c_int64), ("psi_off", c_int64), ("snap_off", c_int64), ("snap_every", c_int64),
                ("n_snap", c_int64), ("tmin", c_double), ("gate_floor", c_double), ("ckpt_off", c_int64),
                ("ckpt_every", c_int64)]


class BufRec(Structure):
    _fields_ = [("fields", c_void_p), ("outputs", c_void_p), ("psi_final", c_void_p), ("snapshots", c_void_p),
                ("counter", c_void_p), ("scratch", c_void_p), ("scratch_bytes", c_size_t)]


class MMAStatusError(RuntimeError):
    pass


_STATUS = {1: "invalid argument", 2: "ground state not converged", 3: "CUDA error", 4: "DFT plan error",
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
    lib.mma_tdse_propagate_ex.argtypes = [c_void_p, c_int, c_void_p, POINTER(BufRec), c_int, c_int, c_int, c_int,
                                          c_void_p]
    lib.mma_tdse_propagate_ex.restype = c_int
    lib.mma_tdse_c64_shape_ok.argtypes = [c_int, c_int]
    lib.mma_tdse_c64_shape_ok.restype = c_int
    lib.mma_tdse_scratch_bytes.argtypes = [c_int, c_int, c_int]
    lib.mma_tdse_scratch_bytes.restype = c_size_t
    lib.mma_tdse_default_ctas.argtypes = [c_int, c_int]
    lib.mma_tdse_default_ctas.restype = c_int
    lib.mma_tdse_c64_default_ctas.argtypes = [c_int, c_int]
    lib.mma_tdse_c64_default_ctas.restype = c_int
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

    ``c64_threads`` (complex64 form only): CTA size the complex64 tables are laid out for --
    None or 256 (every grid), 512 or 1024 (grids that fit that shape, others 256), a list (per
    grid), or "auto" (the autotuner's choice per grid size, mma_gb300.autotune).

    ``df64``: also build the float-float form's tables (the FP64 solve tables split into
    (hi, lo) float pairs) for ``precision="df64"``.
    """

    def __init__(self, params, dt, device="cuda", stream=None, c64=False, adjoint=False, c64_threads=None,
                 df64=False):
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
        self.adjoint = bool(adjoint)
        if self.adjoint:  # A^H solve tables (10 L doubles per grid)
            a_sizes = 10 * THREADS * self.m
            self.adj_buf = torch.zeros(int(a_sizes.sum()), dtype=torch.float64, device=self.device)
            a_off = np.concatenate([[0], np.cumsum(a_sizes)])[:-1]
            for r, o in zip(recs, a_off):
                r.adj_tab = self.adj_buf.data_ptr() + 8 * int(o)
        self.c64 = bool(c64)
        self.c64_threads = np.full(len(recs), THREADS, dtype=np.int64)
        if self.c64:
            if self.m32.max() > 48:
                raise ValueError("the complex64 form takes grids of at most 12288 sites")
            if isinstance(c64_threads, str):
                if c64_threads != "auto":
                    raise ValueError("c64_threads must be None, an int, a list or 'auto'")
                from .autotune import choose_c64_threads

                want = [choose_c64_threads(int(n), self.dt, self.params[g], device=self.device)
                        for g, n in enumerate(self.n)]
            elif c64_threads is None or np.isscalar(c64_threads):
                want = [int(c64_threads or THREADS)] * len(recs)
            else:
                want = [int(t) for t in c64_threads]
                if len(want) != len(recs):
                    raise ValueError("one c64_threads entry per grid")
            for g, t in enumerate(want):
                m32 = -(-int(self.n[g]) // t)
                m32 = -(-m32 // 8) * 8
                if t != THREADS and lib.mma_tdse_c64_shape_ok(t, m32):
                    self.c64_threads[g] = t
                    self.m32[g] = m32
            c_sizes = C64_SLOTS * self.c64_threads * self.m32
            self.c64_buf = torch.zeros(int(c_sizes.sum()), dtype=torch.float32, device=self.device)
            c_off = np.concatenate([[0], np.cumsum(c_sizes)])[:-1]
            for r, m32, o, t in zip(recs, self.m32, c_off, self.c64_threads):
                r.m32 = int(m32)
                r.c64_threads = int(t)
                r.c64_tab = self.c64_buf.data_ptr() + 4 * int(o)
        self.df64 = bool(df64)
        if self.df64:  # the FP64 solve tables as (hi, lo) float pairs: 28 L floats per grid
            d_sizes = 2 * CN_SLOTS * THREADS * self.m  # CN_SLOTS doubles per site, each two floats
            self.df_buf = torch.zeros(int(d_sizes.sum()), dtype=torch.float32, device=self.device)
            d_off = np.concatenate([[0], np.cumsum(d_sizes)])[:-1]
            for r, o in zip(recs, d_off):
                r.df_tab = self.df_buf.data_ptr() + 4 * int(o)
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
        if self.df64:
            lib.mma_tdse_build_df_tables.argtypes = [c_void_p, c_void_p, c_int, c_void_p]
            lib.mma_tdse_build_df_tables.restype = c_int
            _check(lib.mma_tdse_build_df_tables(ctypes.c_void_p(self.dev_recs.data_ptr()), ctypes.addressof(arr),
                                                len(recs), st), "mma_tdse_build_df_tables")
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
    """Outputs of a batch.  ``series(i)`` gives instance i's six series, ``spectrum(i)``
    its source-term spectrum; uniform batches also carry [n_inst, ...] views."""

    def series(self, i):
        o, S = self["out_off"][i], self["S"][i]
        blk = self["outputs"][o:o + 6 * (S + 1)].view(6, S + 1)
        return {k: blk[s, :S] for s, k in enumerate(("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval"))}

    def spectrum(self, i):
        g, row = self["spec_index"][i]
        return self["spec_groups"][g]["F"][row]

    def omegagrid(self, i):
        g, _ = self["spec_index"][i]
        return self["spec_groups"][g]["omega"]


SERIES = ("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval")


class TDSEBatchPlan:
    """A batch of TDSE instances with every device buffer allocated once.

    ``launch()`` issues the whole device pipeline -- Fourier interpolation of the
    fields (one batched DFT pair per field length), the persistent propagation kernel
    (the FP64 and float-float kernels take any grid width, so one launch runs the whole
    batch; complex64 batches run one launch per table shape, or, with
    ``c64_one_launch=True`` and 256-thread tables for every grid, one launch of the
    width-dispatching kernel, which is correct but slower: its register-resident widths
    spill more as called functions than as their own kernels), the output spectra (one
    batch per series length) -- on one
    stream, with no host synchronisation, so ``capture()`` can record it as a CUDA
    graph and ``replay()`` re-runs it on new fields written by ``load_fields``.

    Instances are laid out in the outputs grouped by series length (each group is one
    strided spectrum batch) and handed to the device work queue longest first (the
    cost of an instance is sites x steps), which balances uneven batches.
    """

    def __init__(self, grids, n_field, dt_field, grid_ids=None, dt_req=None, tmin=0.0, precision="fp64",
                 spectra=True, psi_final=False, snap_every=0, tmax=None, grid_ctas=0, c64_one_launch=False):
        lib = _sig()
        self.lib = lib
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % list(PRECISIONS))
        self.grids = grids
        dev = grids.device
        self.device = dev
        nf = np.atleast_1d(np.asarray(n_field, dtype=np.int64))
        n_inst = len(nf)
        if n_inst == 0:
            raise ValueError("empty batch")
        if nf.min() < 2:
            raise ValueError("every field needs at least 2 samples")
        self.n_inst, self.nf = n_inst, nf
        k1, dt = refine(dt_field, dt_req if dt_req is not None else grids.dt)
        if abs(dt - grids.dt) > 1e-12 * grids.dt:
            raise ValueError("grids were built for dt=%g but this batch refines to dt=%g" % (grids.dt, dt))
        self.k1, self.dt, self.dt_field = k1, dt, dt_field
        gid = np.zeros(n_inst, dtype=np.int64) if grid_ids is None else np.asarray(grid_ids, dtype=np.int64)
        if gid.shape != (n_inst,) or gid.min() < 0 or gid.max() >= len(grids):
            raise ValueError("grid_ids must index the grids")
        self.gid = gid
        S = n_steps(nf, k1)
        self.S = S
        self.prec = PRECISIONS[precision]
        if self.prec == 1 and not grids.c64:
            raise ValueError("build the grids with c64=True for the complex64 form")
        if self.prec == 2 and not getattr(grids, "df64", False):
            raise ValueError("build the grids with df64=True for the float-float form")
        # raw and refined field buffers, grouped by raw length
        self.len_groups = []
        raw_total = 0
        fld_off = np.zeros(n_inst, dtype=np.int64)
        off = 0
        for L in np.unique(nf):
            idx = np.nonzero(nf == L)[0]
            self.len_groups.append((int(L), idx, raw_total, off))
            for j, i in enumerate(idx):
                fld_off[i] = off + j * k1 * int(L)
            raw_total += len(idx) * int(L)
            off += len(idx) * k1 * int(L)
        self.raw = torch.zeros(raw_total, dtype=torch.float64, device=dev)
        self.fld = torch.zeros(off, dtype=torch.float64, device=dev)
        # output layout grouped by series length
        out_off = np.zeros(n_inst, dtype=np.int64)
        self.s_groups = []
        off = 0
        for s_len in np.unique(S):
            idx = np.nonzero(S == s_len)[0]
            self.s_groups.append((int(s_len), idx, off))
            for j, i in enumerate(idx):
                out_off[i] = off + j * 6 * (int(s_len) + 1)
            off += len(idx) * 6 * (int(s_len) + 1)
        self.out_off = out_off
        self.outputs = torch.zeros(off, dtype=torch.float64, device=dev)
        self.psi_off = np.full(n_inst, -1, dtype=np.int64)
        self.psi_buf = None
        if psi_final:
            sizes = 2 * grids.n[gid]
            self.psi_off = np.concatenate([[0], np.cumsum(sizes)])[:-1]
            self.psi_buf = torch.zeros(int(sizes.sum()), dtype=torch.float64, device=dev)
        self.snap_off = np.full(n_inst, -1, dtype=np.int64)
        self.n_snap = np.zeros(n_inst, dtype=np.int64)
        self.snap_buf = None
        if snap_every:
            self.n_snap = S // snap_every
            sizes = self.n_snap * 2 * grids.n[gid]
            self.snap_off = np.concatenate([[0], np.cumsum(sizes)])[:-1]
            self.snap_buf = torch.zeros(int(sizes.sum()), dtype=torch.float64, device=dev)
        self.gate_floor = np.zeros(n_inst)
        recs = (InstRec * n_inst)()
        for i in range(n_inst):
            r = recs[i]
            r.grid, r.n_steps, r.field_off, r.n_field = int(gid[i]), int(S[i]), int(fld_off[i]), int(k1 * nf[i])
            r.out_off, r.psi_off, r.snap_off = int(out_off[i]), int(self.psi_off[i]), int(self.snap_off[i])
            r.snap_every, r.n_snap = max(int(snap_every), 1), int(self.n_snap[i]) if snap_every else 0
            r.tmin, r.gate_floor = float(tmin), 0.0
            r.ckpt_off, r.ckpt_every = -1, 0
        self.recs = recs
        # propagation launches, longest first within each: one for the FP64 and float-float forms
        # (width-generic kernels); for the complex64 form one per table shape (sites per thread,
        # CTA size), or -- when every grid's tables are laid out for 256 threads and there are
        # several widths -- one launch of the width-dispatching kernel (shape 0)
        cost = grids.n[gid].astype(np.float64) * S
        if self.prec == 1:
            shapes = grids.m32[gid] * 4096 + grids.c64_threads[gid]
            if c64_one_launch and len(np.unique(shapes)) > 1 and np.all(grids.c64_threads[gid] == THREADS):
                shapes = np.zeros(n_inst, dtype=np.int64)
        else:
            shapes = np.zeros(n_inst, dtype=np.int64)
        self.launches = []
        for shape in sorted(np.unique(shapes), reverse=True):
            idx = np.nonzero(shapes == shape)[0]
            idx = idx[np.argsort(-cost[idx], kind="stable")]
            max_m = int(shape) // 4096 if self.prec == 1 else int(grids.m[np.unique(gid[idx])].max())
            cta_threads = (int(shape) % 4096 or THREADS) if self.prec == 1 else 0
            ctas = grid_ctas or (lib.mma_tdse_c64_default_ctas(max_m, cta_threads) if self.prec == 1
                                 else lib.mma_tdse_default_ctas(max_m, self.prec))
            ctas = min(ctas, len(idx))
            sb = int(lib.mma_tdse_scratch_bytes(max_m, ctas, self.prec))
            self.launches.append(dict(idx=idx, max_m=max_m, ctas=ctas, cta_threads=cta_threads,
                                      scratch=torch.empty(max(sb, 8), dtype=torch.uint8, device=dev), sbytes=sb,
                                      counter=torch.zeros(1, dtype=torch.int32, device=dev)))
        self._upload_records()
        # spectra buffers per series length (rows are the instances of the group)
        self.spectra = spectra
        self.spec_groups = []
        self.spec_index = {}
        if spectra:
            for g, (s_len, idx, off) in enumerate(self.s_groups):
                nc = s_len // 2 + 1
                tm = tmax if tmax is not None else (int(nf[idx[0]]) - 1) * dt_field
                fs = torch.zeros(len(idx), 2 * nc, dtype=torch.float64, device=dev)
                self.spec_groups.append(dict(s=s_len, idx=idx, off=off, tmax=tm, fs=fs,
                                             fm=torch.zeros(len(idx), nc, dtype=torch.float64, device=dev),
                                             omega=torch.zeros(nc, dtype=torch.float64, device=dev),
                                             F=torch.view_as_complex(fs.view(len(idx), nc, 2))))
                for row, i in enumerate(idx):
                    self.spec_index[int(i)] = (g, row)
        self.graph = None

    def _upload_records(self):
        for L in self.launches:
            sub = (InstRec * len(L["idx"]))(*[self.recs[i] for i in L["idx"]])
            L["d_insts"] = torch.frombuffer(bytearray(bytes(sub)), dtype=torch.uint8).to(self.device)

    def load_fields(self, fields):
        """Copy the raw fields (a [n_inst, n_f] tensor or a list of 1-D tensors) into the
        plan's device buffer (on the current stream; no host synchronisation)."""
        uniform = torch.is_tensor(fields) and fields.dim() == 2
        rows = [fields[i] for i in range(fields.shape[0])] if uniform else list(fields)
        if len(rows) != self.n_inst:
            raise ValueError("expected %d fields" % self.n_inst)
        if uniform:  # one copy of the whole tensor (asynchronous from pinned host memory), then
            # each length group from it on the device: a slice when its instances are consecutive
            src = fields.to(self.device, torch.float64, non_blocking=True)
        for L, idx, raw_off, _ in self.len_groups:
            dst = self.raw[raw_off:raw_off + len(idx) * L].view(len(idx), L)
            if uniform:
                i0 = int(idx[0])
                if np.array_equal(np.asarray(idx), np.arange(i0, i0 + len(idx))):
                    dst.copy_(src[i0:i0 + len(idx)], non_blocking=True)
                else:
                    dst.copy_(src[torch.as_tensor(idx, device=self.device)], non_blocking=True)
            else:
                for j, i in enumerate(idx):
                    if rows[i].numel() != L:
                        raise ValueError("field %d has the wrong length" % i)
                    dst[j].copy_(rows[i].to(self.device, torch.float64), non_blocking=True)
        if self.k1 > 1:  # round-off floor of the zero gate after a genuine interpolation
            changed = False
            for L, idx, raw_off, _ in self.len_groups:
                mx = self.raw[raw_off:raw_off + len(idx) * L].view(len(idx), L).abs().amax(dim=1).cpu().numpy()
                for j, i in enumerate(idx):
                    v = 1e-13 * float(mx[j])
                    if self.recs[i].gate_floor != v:
                        self.recs[i].gate_floor = v
                        changed = True
            if changed:
                self._upload_records()

    def check_fields(self):
        if not bool(torch.isfinite(self.raw).all()):
            raise ValueError("field has non-finite samples")

    def launch(self, stream=None, _events=None):
        """Issue the device pipeline on `stream` (default: the current stream)."""
        lib = self.lib
        stream = stream or torch.cuda.current_stream()
        st = ctypes.c_void_p(stream.cuda_stream)
        for L, idx, raw_off, fo in self.len_groups:
            _check(lib.mma_tdse_prepare_fields(self.raw.data_ptr() + 8 * raw_off, len(idx), L, self.k1,
                                               self.fld.data_ptr() + 8 * fo, st), "mma_tdse_prepare_fields")
        if _events is not None:
            _events[0].record(stream)
        for Lc in self.launches:
            B = BufRec(self.fld.data_ptr(), self.outputs.data_ptr(),
                       self.psi_buf.data_ptr() if self.psi_buf is not None else None,
                       self.snap_buf.data_ptr() if self.snap_buf is not None else None, Lc["counter"].data_ptr(),
                       Lc["scratch"].data_ptr(), Lc["sbytes"])
            _check(lib.mma_tdse_propagate_ex(Lc["d_insts"].data_ptr(), len(Lc["idx"]),
                                             self.grids.dev_recs.data_ptr(), ctypes.byref(B), Lc["max_m"],
                                             Lc["cta_threads"], Lc["ctas"], self.prec, st),
                   "mma_tdse_propagate_ex")
        if _events is not None:
            _events[1].record(stream)
        for G in self.spec_groups:
            s = G["s"]
            nc = s // 2 + 1
            _check(lib.mma_tdse_spectra(self.outputs.data_ptr() + 8 * (G["off"] + 2 * (s + 1)), 6 * (s + 1),
                                        len(G["idx"]), s, self.dt, G["tmax"], G["fs"].data_ptr(), 2 * nc,
                                        G["fm"].data_ptr(), nc, G["omega"].data_ptr(), st), "mma_tdse_spectra")

    def capture(self):
        """Record launch() as a CUDA graph (after one eager run that creates the DFT plans)."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch(s)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def result(self):
        res = BatchResult(outputs=self.outputs, out_off=self.out_off, S=self.S, k1=self.k1, dt=self.dt,
                          n_field=self.nf, psi_off=self.psi_off, psi_final=self.psi_buf, snapshots=self.snap_buf,
                          snap_off=self.snap_off, n_snap=self.n_snap, grid_ids=self.gid,
                          ctas=[L["ctas"] for L in self.launches], spec_groups=self.spec_groups,
                          spec_index=self.spec_index)
        if len(self.s_groups) == 1:
            s_len, idx, off = self.s_groups[0]
            if np.array_equal(idx, np.arange(self.n_inst)):
                blk = self.outputs.view(self.n_inst, 6, s_len + 1)
                for j, k in enumerate(SERIES):
                    res[k] = blk[:, j, :s_len]
                if self.spectra:
                    G = self.spec_groups[0]
                    res["Fsourceterm"], res["FsourcetermM2"], res["omegagrid"] = G["F"], G["fm"], G["omega"]
        return res


def run_batch(grids, fields, dt_field, grid_ids=None, dt_req=None, tmin=0.0, spectra=True, psi_final=False,
              snap_every=0, precision="fp64", grid_ctas=0, stream=None, tmax=None, _events=None):
    """Propagate a batch of instances (one-shot form of TDSEBatchPlan).

    fields: float64 cuda tensor [n_inst, n_f] (uniform) or a list of 1-D tensors
    (uneven lengths).  grid_ids: per-instance grid index (default all 0).
    Returns a BatchResult with packed ``outputs``; for uniform batches also views
    ``sourceterm``, ``PopTot``, ``PopInt``, ``expval``, ``Efield``, ``tgrid``
    [n_inst, S] and spectra ``Fsourceterm`` [n_inst, S//2+1] (complex128),
    ``FsourcetermM2``, ``omegagrid``.
    """
    uniform = torch.is_tensor(fields) and fields.dim() == 2
    nf = [fields.shape[1]] * fields.shape[0] if uniform else [int(f.numel()) for f in fields]
    plan = TDSEBatchPlan(grids, nf, dt_field, grid_ids=grid_ids, dt_req=dt_req, tmin=tmin, precision=precision,
                         spectra=spectra, psi_final=psi_final, snap_every=snap_every, tmax=tmax, grid_ctas=grid_ctas)
    plan.load_fields(fields)
    plan.check_fields()
    plan.launch(stream, _events=_events)
    res = plan.result()
    res["_plan"] = plan
    return res
