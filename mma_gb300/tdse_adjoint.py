"""Gradient of a harmonic yield with respect to the driving field (the differentiable form).

For each instance the loss is the reference's spectral intensity summed over a band,

    L = sum_{w_lo <= w_q <= w_hi} FsourcetermM2_q = dt^2/(2 pi) sum_q |DFT_q(sourceterm)|^2

(1DTDSE/sources/tools_fftw3.c:103-132), and ``yield_and_grad`` returns L and dL/dE for
every field sample, by a hand-written adjoint of the FP64 Crank-Nicolson-Numerov step
(mma_gb300/csrc/tdse_adjoint.cu): one forward pass storing the wavefunction every
``ckpt_every`` steps, then, segment by segment from the end, a forward recompute and the
backward adjoint sweep.  ``TDSEYield`` wraps it as a torch.autograd.Function.

The field enters the propagation through the reference's zero gate (prop.c:125-134):
samples up to the gate index are held at 0, so their gradient is 0.  Fields must be
sampled at the propagation step (k1 = 1, no Fourier refinement).
"""
import ctypes
from ctypes import POINTER, c_double, c_int, c_int64, c_size_t, c_void_p

import numpy as np
import torch

from .tdse_batch import BufRec, InstRec, TDSEGrids, _check, _sig, _stream_ptr, n_steps, refine


def _adj_sig():
    lib = _sig()
    if getattr(lib, "_mma_adj_sig", False):
        return lib
    lib.mma_tdse_loss_grad.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_double, c_double, c_double, c_void_p,
                                       c_void_p, c_void_p, c_void_p]
    lib.mma_tdse_loss_grad.restype = c_int
    lib.mma_tdse_adjoint_scratch_bytes.argtypes = [c_int, c_int, c_int]
    lib.mma_tdse_adjoint_scratch_bytes.restype = c_size_t
    lib.mma_tdse_adjoint.argtypes = [c_void_p, c_int, c_void_p, POINTER(BufRec), c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_int, c_int, c_int, c_void_p]
    lib.mma_tdse_adjoint.restype = c_int
    lib._mma_adj_sig = True
    return lib


def gate_indices(fields):
    """The reference's zero-gate index per row (first k with f[k] f[k+1] <= 0, prop.c:125-134)."""
    f = fields.detach()
    nxt = torch.cat([f[:, 1:], torch.zeros_like(f[:, :1])], dim=1)
    hit = (f * nxt) <= 0
    idx = torch.argmax(hit.to(torch.int8), dim=1)
    return idx.cpu().numpy()


def yield_and_grad(grids, fields, dt_field, band, grid_ids=None, ckpt_every=256, tmax=None, want_grad=True):
    """fields: float64 cuda tensor [n_inst, n_f]; band = (w_lo, w_hi) in a.u.
    Returns (L [n_inst], dL/dE [n_inst, n_f] or None) as cuda tensors."""
    lib = _adj_sig()
    dev = grids.device
    if not (torch.is_tensor(fields) and fields.dim() == 2):
        raise ValueError("fields must be a 2-D tensor")
    n_inst, nf = fields.shape
    k1, dt = refine(dt_field, grids.dt)
    if k1 != 1:
        raise NotImplementedError("the adjoint needs fields sampled at the propagation step (k1 = 1)")
    if want_grad and not grids.adjoint:
        raise ValueError("build the grids with adjoint=True")
    gid = np.zeros(n_inst, dtype=np.int64) if grid_ids is None else np.asarray(grid_ids, dtype=np.int64)
    S = int(n_steps(nf, 1))
    K = int(max(1, min(ckpt_every, S)))
    nseg = (S + K - 1) // K
    n_site = grids.n[gid]
    fld = fields.to(dev, torch.float64).contiguous()
    out = torch.zeros(n_inst * 6 * (S + 1), dtype=torch.float64, device=dev)
    ck_sizes = nseg * 2 * n_site
    ck_off = np.concatenate([[0], np.cumsum(ck_sizes)])[:-1]
    ckpts = torch.zeros(int(ck_sizes.sum()), dtype=torch.float64, device=dev)
    recs = (InstRec * n_inst)()
    for i in range(n_inst):
        r = recs[i]
        r.grid, r.n_steps, r.field_off, r.n_field = int(gid[i]), S, i * nf, nf
        r.out_off, r.psi_off, r.snap_off, r.snap_every, r.n_snap = i * 6 * (S + 1), -1, -1, 1, 0
        r.tmin, r.gate_floor = 0.0, 0.0
        r.ckpt_off, r.ckpt_every = int(ck_off[i]), K
    d_recs = torch.frombuffer(bytearray(bytes(recs)), dtype=torch.uint8).to(dev)
    max_m = int(grids.m[np.unique(gid)].max())
    st = _stream_ptr()
    ctas = min(lib.mma_tdse_default_ctas(max_m, 0), n_inst)
    sb = int(lib.mma_tdse_scratch_bytes(max_m, ctas, 0))
    scratch = torch.empty(max(sb, 8), dtype=torch.uint8, device=dev)
    counter = torch.zeros(1, dtype=torch.int32, device=dev)
    B = BufRec(fld.data_ptr(), out.data_ptr(), None, ckpts.data_ptr(), counter.data_ptr(), scratch.data_ptr(), sb)
    _check(lib.mma_tdse_propagate(d_recs.data_ptr(), n_inst, grids.dev_recs.data_ptr(), ctypes.byref(B), max_m, ctas,
                                  0, st), "mma_tdse_propagate")
    tm = torch.full((n_inst,), float(tmax if tmax is not None else (nf - 1) * dt_field), dtype=torch.float64,
                    device=dev)
    loss = torch.zeros(n_inst, dtype=torch.float64, device=dev)
    a = torch.zeros(n_inst * (S + 1), dtype=torch.float64, device=dev)
    a_off = torch.as_tensor(np.arange(n_inst, dtype=np.int64) * (S + 1), device=dev)
    _check(lib.mma_tdse_loss_grad(d_recs.data_ptr(), n_inst, out.data_ptr(), tm.data_ptr(), dt, float(band[0]),
                                  float(band[1]), loss.data_ptr(), a.data_ptr(), a_off.data_ptr(), st),
           "mma_tdse_loss_grad")
    if not want_grad:
        return loss, None
    grad = torch.zeros(n_inst, S, dtype=torch.float64, device=dev)
    g_off = torch.as_tensor(np.arange(n_inst, dtype=np.int64) * S, device=dev)
    actas = min(ctas, n_inst)
    asb = int(lib.mma_tdse_adjoint_scratch_bytes(max_m, K, actas))
    ascratch = torch.empty(asb, dtype=torch.uint8, device=dev)
    B2 = BufRec(fld.data_ptr(), out.data_ptr(), None, ckpts.data_ptr(), counter.data_ptr(), ascratch.data_ptr(), asb)
    _check(lib.mma_tdse_adjoint(d_recs.data_ptr(), n_inst, grids.dev_recs.data_ptr(), ctypes.byref(B2), a.data_ptr(),
                                a_off.data_ptr(), grad.data_ptr(), g_off.data_ptr(), max_m, K, actas, st),
           "mma_tdse_adjoint")
    gE = grad[:, :nf].clone()  # F_k = E_k for k < n_f (k1 = 1); later steps use F = 0
    gate = gate_indices(fld)
    col = torch.arange(nf, device=dev)[None, :]
    gE = torch.where(col <= torch.as_tensor(gate, device=dev)[:, None], torch.zeros_like(gE), gE)
    return loss, gE


class TDSEYield(torch.autograd.Function):
    """loss = TDSEYield.apply(fields, grids, dt_field, (w_lo, w_hi), ckpt_every): per-instance
    band yield, differentiable with respect to the field samples."""

    @staticmethod
    def forward(ctx, fields, grids, dt_field, band, ckpt_every=256):
        loss, g = yield_and_grad(grids, fields, dt_field, band, ckpt_every=ckpt_every,
                                 want_grad=fields.requires_grad)
        ctx.save_for_backward(g if g is not None else torch.zeros(0))
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        (g,) = ctx.saved_tensors
        return grad_loss[:, None] * g, None, None, None, None
