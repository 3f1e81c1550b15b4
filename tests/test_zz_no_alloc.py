"""The allocation-free propagation entry point, called through the C-ABI.

Some hosts cannot call cudaMalloc: their device memory is owned by another
runtime's allocator, or they must not allocate while a graph is recorded.
mma_tdse_propagate_noalloc serves them with a fixed work-space array inside the
library.  This test checks that, on two calls in a row (the array keeps the
previous call's contents), it gives the same results as mma_tdse_propagate with a
caller-provided scratch buffer, within the FP64 parity tolerance of the other
TDSE tests; and that a grid too large for the array is refused without a launch.
This file is named to be collected last.
"""
import ctypes
from ctypes import POINTER, c_int, c_size_t, c_void_p

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-8


def _setup():
    from mma_gb300 import load
    from mma_gb300.tdse_batch import BufRec, InstRec, TDSEGrids, n_steps

    lib = load()
    lib.mma_tdse_propagate_noalloc.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                               c_int, c_void_p]
    lib.mma_tdse_propagate_noalloc.restype = c_int
    lib.mma_tdse_noalloc_capacity_bytes.argtypes = []
    lib.mma_tdse_noalloc_capacity_bytes.restype = c_size_t
    lib.mma_tdse_propagate.argtypes = [c_void_p, c_int, c_void_p, POINTER(BufRec), c_int, c_int, c_int, c_void_p]
    lib.mma_tdse_propagate.restype = c_int
    lib.mma_tdse_scratch_bytes.argtypes = [c_int, c_int, c_int]
    lib.mma_tdse_scratch_bytes.restype = c_size_t

    dt = 0.25
    grids = TDSEGrids([dict(num_r=700, dx=0.3, trg_a=np.sqrt(1.68)), dict(num_r=1500, dx=0.2, trg_a=1.0)], dt=dt)
    rng = np.random.default_rng(11)
    n_inst, nf = 6, 500
    t = dt * np.arange(1, nf + 1)
    T = t[-1] + dt
    fields = np.stack([rng.uniform(0.03, 0.07) * np.sin(np.pi * t / T) ** 2 *
                       np.cos(0.057 * t + rng.uniform(0, 6.28)) for _ in range(n_inst)])
    S = n_steps(nf, 1)
    insts = (InstRec * n_inst)()
    for i in range(n_inst):
        r = insts[i]
        r.grid, r.n_steps, r.field_off, r.n_field = i % 2, S, i * nf, nf
        r.out_off, r.psi_off, r.snap_off, r.snap_every, r.n_snap = i * 6 * (S + 1), -1, -1, 1, 0
        r.tmin, r.gate_floor = 0.0, 0.0
    d_insts = torch.frombuffer(bytearray(bytes(insts)), dtype=torch.uint8).cuda()
    d_fields = torch.tensor(fields.reshape(-1), device="cuda")
    max_m = int(grids.m.max())
    return lib, grids, d_insts, d_fields, n_inst, S, max_m, BufRec


def _run_existing(lib, grids, d_insts, d_fields, n_inst, S, max_m, BufRec):
    out = torch.zeros(n_inst * 6 * (S + 1), dtype=torch.float64, device="cuda")
    sb = lib.mma_tdse_scratch_bytes(max_m, 0, 0)
    scratch = torch.empty(int(sb), dtype=torch.uint8, device="cuda")
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    B = BufRec(d_fields.data_ptr(), out.data_ptr(), None, None, counter.data_ptr(), scratch.data_ptr(), int(sb))
    rc = lib.mma_tdse_propagate(d_insts.data_ptr(), n_inst, grids.dev_recs.data_ptr(), ctypes.byref(B), max_m, 0, 0,
                                torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return out


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def test_noalloc_matches_allocating_entry_point_twice(gpu_lib):
    lib, grids, d_insts, d_fields, n_inst, S, max_m, BufRec = _setup()
    assert lib.mma_tdse_noalloc_capacity_bytes() == 8 << 20
    ref = _run_existing(lib, grids, d_insts, d_fields, n_inst, S, max_m, BufRec)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out = torch.full_like(ref, float("nan"))
        rc = lib.mma_tdse_propagate_noalloc(d_insts.data_ptr(), n_inst, grids.dev_recs.data_ptr(),
                                            d_fields.data_ptr(), out.data_ptr(), None, None, max_m, stream)
        assert rc == 0, "call %d returned status %d" % (call, rc)
        torch.cuda.synchronize()
        blk, rblk = out.view(n_inst, 6, S + 1), ref.view(n_inst, 6, S + 1)
        for s in range(6):  # tgrid, Efield, sourceterm, PopTot, PopInt, expval
            assert _rel(blk[:, s], rblk[:, s]) < TOL, (call, s)


def test_noalloc_rejects_grids_beyond_its_limit(gpu_lib):
    lib, grids, d_insts, d_fields, n_inst, S, max_m, BufRec = _setup()
    out = torch.zeros(n_inst * 6 * (S + 1), dtype=torch.float64, device="cuda")
    rc = lib.mma_tdse_propagate_noalloc(d_insts.data_ptr(), n_inst, grids.dev_recs.data_ptr(), d_fields.data_ptr(),
                                        out.data_ptr(), None, None, 4096, torch.cuda.current_stream().cuda_stream)
    assert rc == 5  # MMA_ERR_TOO_LARGE, refused before any launch
