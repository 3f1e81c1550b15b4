"""The allocation-free propagation entry point, called through the C-ABI.

Some hosts cannot call cudaMalloc: their device memory is owned by another
runtime's allocator, or they must not allocate while a graph is recorded.
mma_tdse_propagate_noalloc serves them with a fixed work-space array inside the
library.  These tests check that, on two calls in a row (the array keeps the
previous call's contents), it gives the same results as mma_tdse_propagate with a
caller-provided scratch buffer -- every series, the final wavefunction and the
wavefunction snapshots -- within the FP64 parity tolerance of the other TDSE tests;
that it matches the oracle; that the device's free memory is the same before and
after a call; that a batch of large grids, where the array rather than the SM count
limits the CTAs, still matches; and that a grid too large for the array is refused
without a launch.  This file is named to be collected last.
"""
import ctypes
from ctypes import POINTER, c_int, c_size_t, c_void_p

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-8
SERIES = ("tgrid", "Efield", "sourceterm", "PopTot", "PopInt", "expval")


def _lib():
    from mma_gb300 import load
    from mma_gb300.tdse_batch import BufRec

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
    return lib


class Case:
    """A batch of instances on the given grids: seeded sin^2 pulses of nf samples each;
    instance 0 also writes its final wavefunction and snapshots every snap_every steps."""

    def __init__(self, grid_params, n_inst, nf, seed, snap_every=50):
        from mma_gb300.tdse_batch import InstRec, TDSEGrids, n_steps

        self.dt = 0.25
        self.params = grid_params
        self.grids = TDSEGrids(grid_params, dt=self.dt)
        rng = np.random.default_rng(seed)
        t = self.dt * np.arange(1, nf + 1)
        T = t[-1] + self.dt
        self.t = t
        self.fields = np.stack([rng.uniform(0.03, 0.07) * np.sin(np.pi * t / T) ** 2 *
                                np.cos(0.057 * t + rng.uniform(0, 6.28)) for _ in range(n_inst)])
        S = n_steps(nf, 1)
        self.S, self.n_inst = S, n_inst
        self.gid = np.arange(n_inst) % len(grid_params)
        n0 = int(self.grids.n[self.gid[0]])
        self.n0 = n0
        self.n_snap = S // snap_every
        insts = (InstRec * n_inst)()
        for i in range(n_inst):
            r = insts[i]
            r.grid, r.n_steps, r.field_off, r.n_field = int(self.gid[i]), S, i * nf, nf
            r.out_off, r.psi_off, r.snap_off, r.snap_every, r.n_snap = i * 6 * (S + 1), -1, -1, 1, 0
            r.tmin, r.gate_floor, r.ckpt_off, r.ckpt_every = 0.0, 0.0, -1, 0
        insts[0].psi_off, insts[0].snap_off, insts[0].snap_every, insts[0].n_snap = 0, 0, snap_every, self.n_snap
        self.d_insts = torch.frombuffer(bytearray(bytes(insts)), dtype=torch.uint8).cuda()
        self.d_fields = torch.tensor(self.fields.reshape(-1), device="cuda")
        self.max_m = int(self.grids.m.max())

    def buffers(self):
        return (torch.full((self.n_inst * 6 * (self.S + 1),), float("nan"), dtype=torch.float64, device="cuda"),
                torch.full((2 * self.n0,), float("nan"), dtype=torch.float64, device="cuda"),
                torch.full((self.n_snap * 2 * self.n0,), float("nan"), dtype=torch.float64, device="cuda"))

    def blocks(self, out):
        return out.view(self.n_inst, 6, self.S + 1)


def _run_existing(lib, c):
    from mma_gb300.tdse_batch import BufRec

    out, psi, snap = c.buffers()
    sb = lib.mma_tdse_scratch_bytes(c.max_m, 0, 0)
    scratch = torch.empty(int(sb), dtype=torch.uint8, device="cuda")
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    B = BufRec(c.d_fields.data_ptr(), out.data_ptr(), psi.data_ptr(), snap.data_ptr(), counter.data_ptr(),
               scratch.data_ptr(), int(sb))
    rc = lib.mma_tdse_propagate(c.d_insts.data_ptr(), c.n_inst, c.grids.dev_recs.data_ptr(), ctypes.byref(B),
                                c.max_m, 0, 0, torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return out, psi, snap


def _run_noalloc(lib, c, bufs, max_m=None):
    out, psi, snap = bufs
    return lib.mma_tdse_propagate_noalloc(c.d_insts.data_ptr(), c.n_inst, c.grids.dev_recs.data_ptr(),
                                          c.d_fields.data_ptr(), out.data_ptr(), psi.data_ptr(), snap.data_ptr(),
                                          c.max_m if max_m is None else max_m,
                                          torch.cuda.current_stream().cuda_stream)


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def _compare(c, got, ref, what):
    (out, psi, snap), (rout, rpsi, rsnap) = got, ref
    blk, rblk = c.blocks(out), c.blocks(rout)
    for s, name in enumerate(SERIES):
        assert _rel(blk[:, s], rblk[:, s]) < TOL, (what, name)
    assert _rel(psi, rpsi) < TOL, (what, "psi_final")
    assert _rel(snap, rsnap) < TOL, (what, "snapshots")


@pytest.fixture(scope="module")
def small_case(gpu_lib):
    return Case([dict(num_r=700, dx=0.3, trg_a=np.sqrt(1.68)), dict(num_r=1500, dx=0.2, trg_a=1.0)], n_inst=6,
                nf=500, seed=11)


def test_noalloc_matches_allocating_entry_point_twice(small_case):
    lib, c = _lib(), small_case
    assert lib.mma_tdse_noalloc_capacity_bytes() == 8 << 20
    ref = _run_existing(lib, c)
    for call in range(2):
        got = c.buffers()
        rc = _run_noalloc(lib, c, got)
        assert rc == 0, "call %d returned status %d" % (call, rc)
        torch.cuda.synchronize()
        _compare(c, got, ref, "call %d" % call)


def test_noalloc_matches_oracle(small_case, oracle_built):
    import oracle.tdse as ot

    lib, c = _lib(), small_case
    got = c.buffers()
    assert _run_noalloc(lib, c, got) == 0
    torch.cuda.synchronize()
    blk = c.blocks(got[0]).cpu().numpy()
    for i in (0, 1):
        p = c.params[c.gid[i]]
        x, psi0, _, _ = ot.ground_state(p["num_r"], p["dx"], p["trg_a"], -1.0, 1e-15)
        o = ot.propagate(x, psi0, c.t, c.fields[i], p["dx"], p["trg_a"])
        assert np.array_equal(blk[i, 0, :c.S], o["tgrid"])
        for s, name in enumerate(SERIES[2:], start=2):
            ref = o[name]
            assert np.linalg.norm(blk[i, s, :c.S] - ref) / np.linalg.norm(ref) < TOL, (i, name)
        if i == 0:
            psi = got[1].cpu().numpy()
            assert np.linalg.norm(psi[0::2] + 1j * psi[1::2] - o["psi"]) / np.linalg.norm(o["psi"]) < TOL


def test_noalloc_call_allocates_no_device_memory(small_case):
    lib, c = _lib(), small_case
    got = c.buffers()
    assert _run_noalloc(lib, c, got) == 0  # any one-time set-up happens on this call
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        assert _run_noalloc(lib, c, got) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "free device memory changed by %d bytes" % (free0 - free1)


def test_noalloc_capped_by_its_array(gpu_lib):
    """Grids of 14001 sites (55 sites per thread): one CTA's sweep buffer is 225,280 bytes, so
    the 8 MiB array holds 37 CTAs -- fewer than the SMs and than the 40 instances -- and the
    launch is sized by the array; results still match the allocating entry point."""
    lib = _lib()
    c = Case([dict(num_r=14000, dx=0.1, trg_a=np.sqrt(1.68))], n_inst=40, nf=120, seed=5, snap_every=40)
    assert c.max_m == 55
    assert (lib.mma_tdse_noalloc_capacity_bytes() - 256) // (55 * 256 * 16) == 37
    ref = _run_existing(lib, c)
    got = c.buffers()
    assert _run_noalloc(lib, c, got) == 0
    torch.cuda.synchronize()
    _compare(c, got, ref, "capped launch")


def test_noalloc_rejects_grids_beyond_its_limit(small_case):
    lib, c = _lib(), small_case
    got = c.buffers()
    rc = _run_noalloc(lib, c, got, max_m=4096)
    assert rc == 5  # MMA_ERR_TOO_LARGE, refused before any launch
