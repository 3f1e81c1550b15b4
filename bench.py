"""Benchmark of the microscopic-to-far-field hot path on one GB300 (or N, as replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the configuration the headline metric is quoted on): the batched FP64
TDSE of 2048 instances -- a 64 (r) x 32 (z) synthetic Gaussian focus (w0 = 100 um,
z in [-5, 5] mm, 800 nm, sin^2 envelope, 10 cycles, peak E0 = 0.0534 a.u.) -- on the
soft-Coulomb grid a^2 = 1.68, x in [-400, 400], dx = 0.1 (8001 sites), dt = 0.25
(4412 steps).  One step = the whole batch: ground state cached, fields resident,
propagation + output spectra.  Site-steps = instances x sites x steps.

Prints one JSON line.  Seeded synthetic inputs; no files are read.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TDSE site-steps/s & Hankel TFLOP/s, chosen vs plain form, 1 GB300, at stated err"
A_CONFIG = math.sqrt(1.68)
OMEGA0 = 0.057
FLOPS_PER_SITE_STEP = 72.0  # algorithmic count of one CN-Numerov site update with observables
GPU_LAUNCHES_PER_STEP = 3  # this library's kernels per batch replay: propagation, spectrum staging, spectrum scaling


# ---------------------------------------------------------------------------------- workload
def focus_fields(n_r=64, n_z=32, n_cycles=10, E0=0.0534, dt=0.25, w0=100e-6, lam=800e-9, zmax=5e-3):
    """E(r, z, t) = E0 (w0/w) exp(-r^2/w^2) sin^2(pi t/T) cos(omega0 t - k r^2/(2R) + Gouy),
    phases as the reference's Gaussian-beam helper (shared_python/mynumerics.py:392-403).
    Instance n = kr + kz * n_r (1DTDSE/sources/MPI-TDSE.c:176-178)."""
    T = n_cycles * 2 * np.pi / OMEGA0
    nf = int(T / dt) + 1
    nf += nf % 2
    t = np.linspace(0.0, T, nf)
    r = np.linspace(0.0, 2 * w0, n_r)
    z = np.linspace(-zmax, zmax, n_z)
    zR = np.pi * w0 ** 2 / lam
    k0 = 2 * np.pi / lam
    zz, rr = np.meshgrid(z, r, indexing="ij")  # [kz, kr]
    w = w0 * np.sqrt(1 + (zz / zR) ** 2)
    amp = E0 * (w0 / w) * np.exp(-(rr / w) ** 2)
    phase = -0.5 * k0 * rr ** 2 * zz / (zR ** 2 + zz ** 2) + np.arctan(zz / zR)
    env = np.sin(np.pi * t / T) ** 2
    fields = amp.reshape(-1, 1) * env[None, :] * np.cos(OMEGA0 * t[None, :] + phase.reshape(-1, 1))
    return t, fields


def config3_inputs(device, n_r=512, n_z=256, n_omega=2048, n_rho=256, seed=0):
    """Config-3 far-field inputs: r in [0, 200 um], z in [-5, 5] mm (the last plane is
    dropped by the source provider, 255 planes integrate), omega in [10, 42] omega0 (800 nm),
    rho in [0, 5 mm], D = 1 m; complex64 source exp(-r^2/(50 um)^2) x a comb of odd
    harmonics 11..41 (Lorentzian width 0.3 omega0) with seeded random phases per plane,
    built on the device (2.15 GB)."""
    import torch

    omega0 = OMEGA0 / 2.4188843265857e-17
    rgrid = np.linspace(0.0, 200e-6, n_r)
    zgrid = np.linspace(-5e-3, 5e-3, n_z)
    ogrid = np.linspace(10 * omega0, 42 * omega0, n_omega)
    rho = np.linspace(0.0, 5e-3, n_rho)
    q = np.arange(11, 42, 2)
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 2 * np.pi, size=(n_z, len(q)))
    lor = 1.0 / (1.0 + ((ogrid[None, :] - q[:, None] * omega0) / (0.3 * omega0)) ** 2)
    comb = torch.tensor(np.exp(1j * ph) @ lor, dtype=torch.complex64, device=device)  # [z, omega]
    prof = torch.tensor(np.exp(-(rgrid / 50e-6) ** 2), dtype=torch.float32, device=device)
    S = comb[:, :, None] * prof[None, None, :]
    return zgrid, rgrid, ogrid, rho, S


def config2_instances(n_inst=4096, seed=0, dt=0.25, dx=0.1):
    """Uneven batch: x half-width ~ U[200, 600] a.u. (dx = 0.1), 6..20-cycle sin^2 pulses,
    peak field log-uniform in [0.02, 0.075] a.u., CEP ~ U[0, 2 pi), seeded.  Each instance has
    its own grid.  Fields start one sample after t = 0."""
    rng = np.random.default_rng(seed)
    half = rng.uniform(200.0, 600.0, n_inst)
    cycles = rng.integers(6, 21, n_inst)
    E0 = np.exp(rng.uniform(np.log(0.02), np.log(0.075), n_inst))
    cep = rng.uniform(0.0, 2 * np.pi, n_inst)
    params, fields = [], []
    for i in range(n_inst):
        params.append(dict(num_r=int(round(2 * half[i] / dx)), dx=dx, trg_a=A_CONFIG))
        T = cycles[i] * 2 * np.pi / OMEGA0
        n = int(T / dt)
        n += n % 2
        t = dt * np.arange(1, n + 1)
        fields.append(E0[i] * np.sin(np.pi * t / T) ** 2 * np.cos(OMEGA0 * t + cep[i]))
    return params, fields, E0


def run_config2(args, device):
    """The uneven batch in the float-float, complex64 and FP64 forms (one plan each); throughput of
    each over three graph replays, and the plateau (H11-H41) error of the two fast forms against
    FP64 per instance."""
    import torch

    from mma_gb300.tdse_batch import TDSEBatchPlan, TDSEGrids

    n_inst = 4096 if args.workload in ("config2", "config1") else 256
    params, fields, E0 = config2_instances(n_inst)
    t0 = time.perf_counter()
    # 256-thread complex64 tables for every grid, so that the one-launch variant takes every width
    grids = TDSEGrids(params, dt=0.25, c64=True, df64=True)
    torch.cuda.synchronize()
    t_grids = time.perf_counter() - t0
    tf = [torch.tensor(f, device=device) for f in fields]
    out = {"instances": n_inst, "grid_build_s": t_grids, "site_steps": float(sum(
        (p["num_r"] + 1) * (len(f) + 2) for p, f in zip(params, fields)))}
    res = {}
    for prec in ("df64", "c64", "c64_one_launch", "fp64"):
        plan = TDSEBatchPlan(grids, [len(f) for f in fields], 0.25, grid_ids=np.arange(n_inst),
                             precision="c64" if prec == "c64_one_launch" else prec,
                             c64_one_launch=prec == "c64_one_launch")
        plan.load_fields(tf)
        plan.capture()  # one eager run (DFT plans), then the graph
        if prec != "fp64":  # the FP64 form (18 s a batch) is timed on its first replay
            plan.replay()
        torch.cuda.synchronize()
        reps = 3 if prec != "fp64" else 1
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in ev:
            e0.record()
            plan.replay()
            e1.record()
        torch.cuda.synchronize()
        secs = [a.elapsed_time(b) * 1e-3 for a, b in ev]
        sec = float(np.median(secs))
        out[prec] = {"seconds": sec, "replays": reps, "site_steps_per_s": out["site_steps"] / sec,
                     "propagation_launches": len(plan.launches)}
        res[prec] = plan
    # plateau error per instance (FP64 form = the oracle's arithmetic, checked by the tests)
    ref = res["fp64"].result()
    for prec in ("df64", "c64"):
        rr = res[prec].result()
        errs = []
        for i in range(n_inst):
            a = rr.spectrum(i)
            b = ref.spectrum(i)
            om = ref.omegagrid(i)
            sel = (om >= 11 * OMEGA0) & (om <= 41 * OMEGA0)
            pa, pb = a[sel].abs() ** 2, b[sel].abs() ** 2
            errs.append(float(torch.linalg.norm(pa - pb) / torch.linalg.norm(pb)))
        errs = np.array(errs)
        out[prec]["speedup_vs_fp64"] = out["fp64"]["seconds"] / out[prec]["seconds"]
        out[prec]["plateau_rel_err"] = {"median": float(np.median(errs)), "p90": float(np.percentile(errs, 90)),
                                        "max": float(errs.max()),
                                        "median_E0_ge_0.04": float(np.median(errs[E0 >= 0.04]))}
    return out


def run_config0(args, device):
    """Config 0: one 8001-site instance (10-cycle 800 nm sin^2 pulse, E0 = 0.0534 a.u.) through the
    PythonCTDSE surface -- the legacy C-ABI in the FP64 plain form, ground state, propagation and
    spectra, host arrays in and out -- timed wall-clock per call; the same instance in the
    float-float form through the batched API; and the oracle port on one host core.  The field is
    the one the reference DLL was run on for tests/golden/tdse_config0.npz, so each form's
    relative L2 error against the reference's own outputs is reported beside its time."""
    import torch

    from mma_gb300.tdse import TDSE_DLL, run_single
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "tdse_config0.npz"))
    t, E = g["t"], g["E"]
    num_r, dx, a = int(g["params"][0]), float(g["params"][1]), float(g["params"][2])
    series = ("sourceterm", "PopTot", "PopInt", "expval", "Fsourceterm")

    def errs(res):
        return {k: float(np.linalg.norm(np.asarray(res[k]) - g[k]) / np.linalg.norm(g[k])) for k in series}

    dll = TDSE_DLL()
    run_single(dll, t, E, num_r=num_r, dx=dx, trg_a=a, CV=1e-15)  # warm-up (DFT plan, module load)
    secs = []
    for _ in range(3):
        t0 = time.perf_counter()
        r = run_single(dll, t, E, num_r=num_r, dx=dx, trg_a=a, CV=1e-15)
        secs.append(time.perf_counter() - t0)
    site_steps = float((num_r + 1) * r["Nt"])
    out = {"instances": 1, "sites": num_r + 1, "steps": int(r["Nt"]), "site_steps": site_steps,
           "legacy_fp64": {"seconds_per_call": float(np.median(secs)), "calls": len(secs),
                           "site_steps_per_s": site_steps / float(np.median(secs)),
                           "rel_l2_vs_reference": errs(r),
                           "note": "wall clock of the PythonCTDSE-surface call: ground state, one CTA "
                                   "propagating, spectra, host copies"}}
    dtf = float(t[1] - t[0])
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=a)], dt=dtf, df64=True)
    Ed = torch.tensor(E[None, :], device=device)
    for prec in ("fp64", "df64"):
        run_batch(grids, Ed, dt_field=dtf, tmax=float(t[-1] - t[0]), precision=prec)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        res = run_batch(grids, Ed, dt_field=dtf, tmax=float(t[-1] - t[0]), precision=prec)
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3
        host = {k: res[k][0].cpu().numpy() for k in series}
        out["batch_" + prec] = {"seconds": sec, "site_steps_per_s": site_steps / sec,
                                "rel_l2_vs_reference": errs(host)}
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        _cpu_instance(("port", None, t, E, num_r, dx, a))
        cpu = time.perf_counter() - t0
        out["cpu_port_1_core"] = {"seconds": cpu, "site_steps_per_s": site_steps / cpu,
                                  "note": "the oracle's C restatement, one instance on one host core"}
        out["legacy_speedup_vs_1_core"] = cpu / out["legacy_fp64"]["seconds_per_call"]
    return out


def run_config4(args, device):
    """Adjoint: 256 instances on the config-1 grid (every 8th instance of the config-1 focus),
    L = harmonic yield over [21, 31] omega0, checkpoints every 256 steps; timing of the
    forward + adjoint gradient against the forward alone, and central finite differences
    (h = 1e-6 a.u.) at 32 random samples per instance (each finite-difference pass perturbs
    one sample in every instance: the instances are independent)."""
    import torch

    from mma_gb300.tdse_adjoint import yield_and_grad
    from mma_gb300.tdse_batch import TDSEGrids

    n_inst = 256 if args.workload in ("config4", "config1") else 16
    t, fields_np = focus_fields()
    fields = torch.tensor(fields_np[::len(fields_np) // n_inst][:n_inst], device=device)
    dtf = t[1] - t[0]
    band = (21 * OMEGA0, 31 * OMEGA0)
    grids = TDSEGrids([dict(num_r=8000, dx=0.1, trg_a=A_CONFIG)], dt=dtf, adjoint=True)
    yield_and_grad(grids, fields[:2], dtf, band)  # warm-up
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e[0].record()
    L0, _ = yield_and_grad(grids, fields, dtf, band, want_grad=False)
    e[1].record()
    L, g = yield_and_grad(grids, fields, dtf, band, ckpt_every=256)
    e[2].record()
    torch.cuda.synchronize()
    t_fwd, t_grad = e[0].elapsed_time(e[1]) * 1e-3, e[1].elapsed_time(e[2]) * 1e-3
    n_samples = getattr(args, "fd_samples", None) or (32 if args.workload == "config4" else 4)
    rng = np.random.default_rng(0)
    nf = fields.shape[1]
    idx = np.stack([rng.choice(np.arange(4, nf - 4), size=n_samples, replace=False) for _ in range(n_inst)])
    h = 1e-6
    fd = np.zeros((n_inst, n_samples))
    rows = torch.arange(n_inst, device=device)
    for j in range(n_samples):
        cols = torch.as_tensor(idx[:, j], device=device)
        fp = fields.clone()
        fm = fields.clone()
        fp[rows, cols] += h
        fm[rows, cols] -= h
        Lp, _ = yield_and_grad(grids, fp, dtf, band, want_grad=False)
        Lm, _ = yield_and_grad(grids, fm, dtf, band, want_grad=False)
        fd[:, j] = ((Lp - Lm) / (2 * h)).cpu().numpy()
    gn = g.cpu().numpy()
    ga = np.take_along_axis(gn, idx, axis=1)
    scale = np.abs(gn).max(axis=1, keepdims=True)
    err = np.abs(ga - fd) / scale
    return {"instances": n_inst, "steps": int(nf + 2), "sites": 8001, "checkpoint_every": 256,
            "band_omega0": [21, 31], "forward_s": t_fwd, "forward_plus_adjoint_s": t_grad,
            "gradient_cost_in_forwards": t_grad / t_fwd,
            "site_steps_per_s_gradient": n_inst * 8001.0 * (nf + 2) / t_grad,
            "fd": {"h": h, "samples_per_instance": n_samples,
                   "max_abs_err_over_max_grad": float(err.max()), "median": float(np.median(err))},
            "loss_matches_forward": float(torch.max(torch.abs(L - L0) / L0))}


HANKEL_FLOP_PER_TERM = 8.0  # one complex multiply-accumulate per (omega, plane, rho, r) term


def run_hankel(args, device):
    import torch

    from mma_gb300 import hankel as H

    H.set_stage1_form(getattr(args, "stage1", "cuda"))
    H.XUV_index.set_constant_index(complex(1 - 1e-5, 1e-7))
    zgrid, rgrid, ogrid, rho, S = config3_inputs(device, n_omega=WORKLOADS[args.workload][3])
    target = H.FSources_provider(zgrid, rgrid, ogrid, FSource=S, device=device)
    del S
    z = target.zgrid
    pre, _ = H.pre_factor_table(z, target.ogrid, "Ar", 1.0)
    pre_d = torch.as_tensor(pre, device=device)  # resident like the source (the e2e pass uploads the host table)
    Nz, No, Nr = target.source.shape
    terms = float(No) * Nz * len(rho) * Nr
    stream = torch.cuda.current_stream()
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=device)

    def run(form, planes=(0, -1)):
        return H.far_field(target.ogrid, target.rgrid, z, rho, target.source, 1.0, pre_d, True, planes=planes,
                           form=form, tol=getattr(args, "ff_tol", 1e-9))

    out = {}
    for _ in range(max(args.warmup, 3)):
        run("fast")
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.add_(1.0)
        ev[i][0].record(stream)
        ff_fast, _, plan = run("fast")
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    t_fast = float(np.mean([a.elapsed_time(b) for a, b in ev])) * 1e-3
    # the same far field recorded once as a CUDA graph and replayed (no host work per call)
    ffp = H.FarFieldPlan(target.ogrid, target.rgrid, z, rho, target.source, 1.0, pre_d, True, planes=(0, -1),
                         tol=getattr(args, "ff_tol", 1e-9))
    evg = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.add_(1.0)
        evg[i][0].record(stream)
        ffg, _ = ffp.replay()
        evg[i][1].record(stream)
    torch.cuda.synchronize()
    t_graph = float(np.mean([a.elapsed_time(b) for a, b in evg])) * 1e-3
    graph_same = bool(torch.equal(ffg, ff_fast))
    del ffp
    # plain FP64: one warm-up on a 32-frequency slice, then one timed full far field
    sl = H.FSources_provider(np.append(z, z[-1] + (z[-1] - z[-2])), target.rgrid, target.ogrid[:32],
                             FSource=target.source[:, :32].clone(), device=device)
    H.far_field(sl.ogrid, sl.rgrid, sl.zgrid, rho, sl.source, 1.0, pre[:, :32], True, form="plain")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.add_(1.0)
    e0.record(stream)
    ff_plain, _, _ = run("plain")
    e1.record(stream)
    torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) * 1e-3
    a = ff_fast.cpu().numpy()
    b = ff_plain.cpu().numpy()
    ph = np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)
    # end to end through the public API: pinned host source in, host far field out
    # (two untimed passes, then the median of three timed ones)
    host_src = target.source.cpu().pin_memory()
    host_ff = torch.empty(len(rho), No, dtype=torch.complex128).pin_memory()
    t_runs = []
    for it in range(5):
        e0.record(stream)
        # the public call on the pinned host source: blocks of frequencies are uploaded on a
        # second stream while the blocks already on the device are computed
        ffe, _, _ = H.far_field(target.ogrid, target.rgrid, z, rho, host_src, 1.0, pre, True, planes=(0, -1),
                                form="fast", tol=getattr(args, "ff_tol", 1e-9))
        host_ff.copy_(ffe, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        if it >= 2:
            t_runs.append(e0.elapsed_time(e1) * 1e-3)
        del ffe
    t_e2e = float(np.median(t_runs))
    h2d_bytes, d2h_bytes = host_src.numel() * 8, host_ff.numel() * 16
    del host_src
    allp = run_all_planes(args, target, z, rho, pre_d, flush, stream)
    out = {"workload": "config3: N_r=512, N_z=256 (255 planes integrated), N_omega=2048, N_rho=256, D=1 m, "
                       "complex64 source, constant XUV index n=1-1e-5+1e-7i, near-field factor on",
           "terms": terms, "flop_per_term": HANKEL_FLOP_PER_TERM,
           "plain_fp64": {"seconds": t_plain, "tflops_algorithmic": HANKEL_FLOP_PER_TERM * terms / t_plain / 1e12},
           "chosen_fast": {"seconds": t_fast, "tflops_algorithmic": HANKEL_FLOP_PER_TERM * terms / t_fast / 1e12,
                           "speedup_vs_plain": t_plain / t_fast, "series_terms": plan["n_terms"],
                           "truncation_bound": plan["trunc_bound"],
                           "per_harmonic_rel_err_vs_plain": {"max": float(ph.max()), "median": float(np.median(ph))},
                           "includes": "FF_integrated plus entry and exit plane transforms"},
           "chosen_fast_graph": {"seconds": t_graph, "tflops_algorithmic": HANKEL_FLOP_PER_TERM * terms / t_graph / 1e12,
                                 "identical_to_call": graph_same,
                                 "what": "hankel.FarFieldPlan replay: the fast form's kernels recorded once as a "
                                         "CUDA graph, without the host's per-call work"},
           "e2e_fast": {"seconds": t_e2e, "h2d_bytes": h2d_bytes, "d2h_bytes": d2h_bytes,
                        "upload": "pinned host source in blocks of %d frequencies on a second stream, each block's "
                                  "fast form running as it lands" % H.STREAM_BLOCK,
                        "tflops_algorithmic": HANKEL_FLOP_PER_TERM * terms / t_e2e / 1e12},
           "all_planes": allp}
    return out


def run_profile_case(args, device):
    """Small cases for kernel captures (one untimed pass each): ``small_wide`` propagates 152
    instances on grids of 9001-12001 sites (the register-resident complex64 kernel, 40 and 48
    sites per thread) with 2-cycle pulses; ``small_adjoint`` runs the adjoint gradient of 16
    config-1-grid instances with 2-cycle pulses."""
    import torch

    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    if args.workload == "small_wide":
        sizes = [9000, 10000, 11000, 12000]
        t, fields = focus_fields(n_r=8, n_z=19, n_cycles=2)
        grids = TDSEGrids([dict(num_r=n, dx=0.1, trg_a=A_CONFIG) for n in sizes], dt=float(t[1] - t[0]), c64=True)
        ids = np.arange(fields.shape[0]) % len(sizes)
        res = run_batch(grids, torch.tensor(fields, device=device), float(t[1] - t[0]), grid_ids=ids,
                        precision="c64", tmax=float(t[-1] - t[0]))
        torch.cuda.synchronize()
        return {"instances": int(fields.shape[0]), "sites_per_thread": sorted(set(int(m) for m in grids.m32)),
                "finite": bool(torch.isfinite(res["sourceterm"]).all())}
    from mma_gb300.tdse_adjoint import yield_and_grad

    t, fields = focus_fields(n_r=4, n_z=4, n_cycles=2)
    dtf = float(t[1] - t[0])
    grids = TDSEGrids([dict(num_r=8000, dx=0.1, trg_a=A_CONFIG)], dt=dtf, adjoint=True)
    L, g = yield_and_grad(grids, torch.tensor(fields, device=device), dtf, (11 * OMEGA0, 21 * OMEGA0), ckpt_every=256)
    torch.cuda.synchronize()
    return {"instances": int(fields.shape[0]), "finite": bool(torch.isfinite(g).all())}


def run_analysis(args, device):
    """Analysis functions of the TDSE library on config-1 sizes: the photoelectron spectrum of
    an 8001-site wavefunction on the reference's default energy grid (10000 energies, window
    5e-4) and the Gabor transforms of 512 config-1 fields (4410 samples, 100 windows, omega <= 2).
    GPU times by CUDA events; the numpy restatement timed on a sample (400 energies, 4 signals)
    as the CPU baseline, extrapolated linearly."""
    import torch

    import oracle.analysis as oa
    from mma_gb300 import analysis

    num_r, dx = 8000, 0.1
    x = np.arange(num_r + 1) * dx - 0.5 * num_r * dx
    rng = np.random.default_rng(0)
    psi = (np.exp(-np.abs(x)) + 0.3 * np.exp(-((x - 40.0) / 10.0) ** 2) * np.exp(1j * 0.9 * x)
           + 0.01 * rng.standard_normal(x.size) * np.exp(-(x / 60.0) ** 2))
    dpsi = torch.tensor(psi, device=device)
    kw = dict(E_start=-0.6, num_E=10000, epsilon=5e-4, Estep=5e-4)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    analysis.pes(dpsi, num_r, dx, A_CONFIG, **kw)
    ts = []
    for _ in range(3):
        e0.record(stream)
        _, P = analysis.pes(dpsi, num_r, dx, A_CONFIG, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t_pes = float(np.median(ts))
    ns = 400
    c0 = time.perf_counter()
    ref = oa.pes(psi, num_r, dx, A_CONFIG, ns, kw["epsilon"], kw["Estep"], kw["E_start"])
    t_cpu_pes = (time.perf_counter() - c0) * kw["num_E"] / ns
    err_pes = float(np.abs(P[:ns].cpu().numpy() - ref).max() / np.abs(ref).max())
    t, fields = focus_fields(n_r=WORKLOADS["config1"][0], n_z=WORKLOADS["config1"][1], n_cycles=10)
    sig = torch.tensor(fields[:512], device=device)
    dt = float(t[1] - t[0])
    gkw = dict(omega_max=2.0, t_min=0.0, t_max=float(t[-1]), N_G=100, a=8.0)
    analysis.gabor(sig, dt, **gkw)
    ts = []
    for _ in range(3):
        e0.record(stream)
        _, om, G = analysis.gabor(sig, dt, **gkw)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t_gab = float(np.median(ts))
    c0 = time.perf_counter()
    refg = [oa.gabor(fields[i], dt, fields.shape[1], len(om), gkw["N_G"], gkw["t_min"], gkw["t_max"], gkw["a"])
            for i in range(4)]
    t_cpu_gab = (time.perf_counter() - c0) * 512 / 4
    Gh = G[:4].cpu().numpy()
    err_gab = float(max(np.abs(Gh[i] - refg[i]).max() / np.abs(refg[i]).max() for i in range(4)))
    return {"pes": {"sites": num_r + 1, "energies": kw["num_E"], "gpu_seconds": t_pes,
                    "cpu_seconds_extrapolated": t_cpu_pes, "cpu_sample": "%d energies, numpy restatement, 1 process" % ns,
                    "speedup": t_cpu_pes / t_pes, "rel_err_vs_oracle": err_pes},
            "gabor": {"signals": 512, "samples": int(fields.shape[1]), "windows": gkw["N_G"], "frequencies": len(om),
                      "gpu_seconds": t_gab, "cpu_seconds_extrapolated": t_cpu_gab,
                      "cpu_sample": "4 signals, numpy restatement, 1 process", "speedup": t_cpu_gab / t_gab,
                      "rel_err_vs_oracle": err_gab}}


def tc_geometry(n_terms, n_omega, n_rho, n_z, n_r):
    """Padded GEMM extents of the tensor-core plane form: rows (rho, m), columns (plane, re/im), inner r."""
    mm = {8: 8, 12: 16, 16: 16, 20: 32, 24: 32, 32: 32}[int(n_terms)]
    rc = 2 * (128 // mm)
    n_rb = -(-n_rho // rc)
    zpad = -(-n_z // 128) * 128
    rpad = -(-n_r // 32) * 32
    rows = n_omega * n_rb * rc * mm
    return {"terms": mm, "rows": rows, "cols": 2 * zpad, "inner": rpad,
            "flops_executed": 2.0 * 3 * rows * 2 * zpad * rpad,
            "flops_useful": 2.0 * 3 * n_omega * n_rho * mm * 2 * n_z * n_r}


def run_all_planes(args, target, z, rho, pre, flush, stream):
    """Every plane transform of config 3 (what Hankel_long's cumulative results need): the
    tensor-core split-precision form (three FP16 GEMM terms per product, FP32 accumulation) against
    the direct FP32 form (one J0 per term) and the plain FP64 form; errors per harmonic and plane
    against the plain form."""
    import torch

    from mma_gb300 import hankel as H

    Nz, No, Nr = target.source.shape
    allp = list(range(Nz))

    def call(form, via="auto", events=None):
        return H.far_field(target.ogrid, target.rgrid, z, rho, target.source, 1.0, pre, True, planes=allp,
                           form=form, planes_via=via, _events=events)

    for _ in range(2):
        call("fast", "tc")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_all, t_k = [], []
    ptc = plan = None
    for _ in range(max(args.steps, 3)):
        ptc = None
        flush.add_(1.0)
        e0.record(stream)
        ff_tc, ptc, plan = call("fast", "tc", (k0, k1))
        e1.record(stream)
        torch.cuda.synchronize()
        t_all.append(e0.elapsed_time(e1) * 1e-3)
        t_k.append(k0.elapsed_time(k1) * 1e-3)
    P_tc = torch.stack([ptc[k] for k in allp])
    del ptc
    flush.add_(1.0)
    e0.record(stream)
    _, pdir, _ = call("fast", "direct")
    e1.record(stream)
    torch.cuda.synchronize()
    t_dir = e0.elapsed_time(e1) * 1e-3
    P_dir = torch.stack([pdir[k] for k in allp])
    del pdir
    flush.add_(1.0)
    e0.record(stream)
    ff64, p64, _ = call("plain")
    e1.record(stream)
    torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) * 1e-3
    P64 = torch.stack([p64[k] for k in allp])
    del p64
    e_ff = (torch.linalg.norm(ff_tc - ff64, dim=0) / torch.linalg.norm(ff64, dim=0)).cpu().numpy()
    nrm = torch.linalg.norm(P64, dim=1)  # [plane, omega]
    e_tc = (torch.linalg.norm(P_tc - P64, dim=1) / nrm).flatten()
    e_dir = (torch.linalg.norm(P_dir - P64, dim=1) / nrm).flatten()
    del P_tc, P_dir, P64
    geo = tc_geometry(plan["n_terms"], No, len(rho), Nz, Nr)
    tk = float(np.median(t_k))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("bf16_tflops")
    ach = geo["flops_executed"] / tk / 1e12
    terms = float(No) * Nz * len(rho) * Nr
    return {"planes": Nz, "tc_series_terms": geo["terms"],
            "tensor_core": {"seconds": float(np.median(t_all)), "kernel_seconds": tk,
                            "tflops_executed": ach, "tflops_useful": geo["flops_useful"] / tk / 1e12,
                            "tflops_algorithmic": HANKEL_FLOP_PER_TERM * terms / float(np.median(t_all)) / 1e12,
                            "roofline": {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                                         "frac": ach / peak if peak else None,
                                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst; FP16 dense "
                                                        "runs at the BF16 rate)"},
                            "gemm": geo,
                            "per_harmonic_rel_err_vs_plain": {"max": float(e_tc.max()),
                                                              "median": float(e_tc.median())},
                            "ff_integrated_via": plan.get("ff_via"),
                            "ff_integrated_per_harmonic_rel_err_vs_plain": {"max": float(e_ff.max()),
                                                                            "median": float(np.median(e_ff))},
                            "includes": "plane tables + B operand + tensor-core kernel + FF_integrated (the z "
                                        "trapezoid of the planes); kernel_seconds is the tensor-core kernel "
                                        "alone"},
            "direct_fp32": {"seconds": t_dir, "per_harmonic_rel_err_vs_plain": {"max": float(e_dir.max()),
                                                                                 "median": float(e_dir.median())}},
            "plain_fp64": {"seconds": t_plain},
            "speedup_tc_vs_direct": t_dir / float(np.median(t_all)),
            "speedup_tc_vs_plain": t_plain / float(np.median(t_all))}


def hankel_cpu_baseline(cores=None):
    """The numpy restatement (oracle) on a slice of config 3 -- 16 frequencies x 9 source
    planes (8 integrated) x 256 rho x 512 r -- split over frequencies on `cores` spawned
    processes, extrapolated linearly in terms to the full far field."""
    import multiprocessing as mp

    cores = cores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_hankel_slice, [(i, cores) for i in range(cores)])
        wall = time.perf_counter() - t0
    terms = sum(res)
    full = 2048.0 * 255 * 256 * 512
    rate = terms / wall
    return {"value": HANKEL_FLOP_PER_TERM * rate / 1e12, "unit": "TFLOP/s (algorithmic)", "cores": cores,
            "kind": "port", "seconds_full_extrapolated": full / rate,
            "sample": "numpy restatement, %d frequencies x 8 planes x 256 rho x 512 r on %d processes, %.1f s; "
                      "extrapolated linearly in terms to config 3" % (8 * cores, cores, wall)}


def _hankel_slice(args):
    i, n = args
    import oracle.hankel as oh

    omega0 = OMEGA0 / 2.4188843265857e-17
    og = np.linspace(10 * omega0, 42 * omega0, 2048)[i::n][:8]
    rg = np.linspace(0.0, 200e-6, 512)
    rho = np.linspace(0.0, 5e-3, 256)
    z = np.linspace(-5e-3, 5e-3, 256)[:10]
    S = np.exp(-(rg / 50e-6) ** 2)[None, None, :] * np.ones((len(z), len(og), 1), dtype=np.complex64)
    oh.hankel_long(z, rg, og, S, 1.0, rho)
    return len(og) * (len(z) - 1) * 256 * 512


# ---------------------------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.split("\n") if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_mhz_min": float(np.min(sm)), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------- CPU baseline
def _cpu_instance(args):
    """One config-1 instance on the CPU (the reference DLL when built, else the oracle port)."""
    kind, ref_path, t, E, num_r, dx, a = args
    t0 = time.perf_counter()
    if kind == "reference":
        from mma_gb300.tdse import TDSE_DLL, run_single

        r = run_single(TDSE_DLL(ref_path), t, E, num_r=num_r, dx=dx, trg_a=a, CV=1e-15)
        steps = r["Nt"]
    else:
        import oracle.tdse as ot

        x, psi0, _, _ = ot.ground_state(num_r, dx, a, -1.0, 1e-15)
        o = ot.propagate(x, psi0, t, E, dx, a)
        steps = o["n_out"]
    return (num_r + 1) * steps, time.perf_counter() - t0


def cpu_baseline(t, fields, n_inst, cores=None):
    """Time n_inst config-1 instances on `cores` worker processes (spawned) of the host."""
    import multiprocessing as mp

    import oracle

    oracle.build(ref=None)
    ref = oracle.ref_dll_path()
    kind = "reference" if ref else "port"
    cores = cores or os.cpu_count() or 1
    jobs = [(kind, ref, t, fields[i % len(fields)], 8000, 0.1, A_CONFIG) for i in range(n_inst)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_cpu_instance, jobs)
        wall = time.perf_counter() - t0
    site_steps = sum(r[0] for r in res)
    return {"value": site_steps / wall, "unit": "site-steps/s", "cores": cores, "kind": kind,
            "sample": "%d config-1 instances (8001 sites x %d steps each) on %d processes, %.1f s wall"
                      % (n_inst, res[0][0] // 8001, cores, wall)}


# ---------------------------------------------------------------------------------- GPU arm
def l2_flush(buf):
    buf.add_(1.0)


WORKLOADS = {
    # name: (n_r, n_z, n_cycles, hankel n_omega)
    "config0": (64, 32, 10, 2048),  # one instance through the PythonCTDSE surface (run_config0)
    "config1": (64, 32, 10, 2048),
    "config2": (64, 32, 10, 2048),  # uneven batch (run_config2), reported on its own line
    "config4": (64, 32, 10, 2048),  # adjoint gradients (run_config4), reported on its own line
    "config3": (64, 32, 10, 2048),  # the far field alone (run_hankel), reported on its own line
    "analysis": (64, 32, 10, 2048),  # photoelectron spectra and Gabor transforms (run_analysis)
    "small": (8, 19, 2, 128),  # profiling case: same grids, fewer instances, shorter pulses
    "small_df": (16, 19, 2, 128),  # profiling case: 304 instances, two float-float CTAs per SM
    "small_wide": (8, 19, 2, 128),  # profiling case: grids of 9001-12001 sites (run_profile_case)
    "small_adjoint": (8, 19, 2, 128),  # profiling case: the adjoint on 16 short pulses (run_profile_case)
    "small_ff": (8, 19, 2, 256),  # profiling case: config-3 far field with 256 frequencies (268 MB source)
}


def max_over_ranks(x, world, device=None):
    """The largest value of x over the ranks, on every rank: the step time of the slowest replica,
    which sets the whole job's throughput.  NCCL reduces on the rank's GPU, other backends on CPU."""
    if world <= 1:
        return float(x)
    import torch

    on_gpu = device is not None and torch.distributed.get_backend() == "nccl"
    tt = torch.tensor([float(x)], dtype=torch.float64, device=device if on_gpu else "cpu")
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(units_per_rank, seconds_slowest, world):
    """Whole-job throughput of `world` independent replicas that each process units_per_rank,
    timed by the slowest replica (weak scaling)."""
    return world * units_per_rank / seconds_slowest


def run_ours(args, rank, world, precision):
    import torch

    from mma_gb300 import load
    from mma_gb300.tdse_batch import TDSEBatchPlan, TDSEGrids, run_batch

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    lib = load()
    wr, wz, wc, _ = WORKLOADS[args.workload]
    t, fields_np = focus_fields(n_r=wr, n_z=wz, n_cycles=wc)
    dtf = t[1] - t[0]
    tmax = t[-1] - t[0]
    n_inst = fields_np.shape[0]
    fields = torch.tensor(fields_np, device=dev)
    grids = TDSEGrids([dict(num_r=8000, dx=0.1, trg_a=A_CONFIG)], dt=dtf, c64=(precision == "c64"),
                      c64_threads=(args.c64_threads if args.c64_threads == "auto" else int(args.c64_threads))
                      if precision == "c64" else None, df64=(precision == "df64"))
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    stream = torch.cuda.current_stream()
    plan = TDSEBatchPlan(grids, [fields.shape[1]] * n_inst, dtf, tmax=tmax, precision=precision)
    plan.load_fields(fields)
    plan.check_fields()
    plan.capture()  # the whole batch (interpolation, propagation, spectra) as one CUDA graph

    def step():
        plan.replay()
        return plan.result()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    S = int(plan.S[0])
    sites = 8001
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        for i in range(args.steps):
            l2_flush(flush)
            ev[i][0].record(stream)
            res = step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    ms_step = max_over_ranks(float(np.mean(ms)), world, dev)
    site_steps = float(n_inst) * sites * S
    value = replica_throughput(site_steps, ms_step * 1e-3, world)

    # end to end through the public API: host (pinned) fields in; back to the host everything
    # the reference's per-instance call returns (outputs_def): the six series tgrid, Efield,
    # sourceterm, PopTot, PopInt, expval, and the source-term spectrum F and |F|^2
    host_fields = torch.tensor(fields_np).pin_memory()
    res0 = plan.result()
    host_series = torch.empty(plan.outputs.shape, dtype=torch.float64).pin_memory()
    host_F = torch.empty(res0["Fsourceterm"].shape, dtype=torch.complex128).pin_memory()
    host_M2 = torch.empty(res0["FsourcetermM2"].shape, dtype=torch.float64).pin_memory()
    # events: start, fields on the device, batch done, results on the host
    e2e_ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e_ms, e_parts = [], []
    clk_e2e = ClockSampler(dev.index)
    clk_e2e.__enter__()
    for it in range(1 + max(2, min(args.steps, 3))):  # the first pass is an untimed warm-up
        l2_flush(flush)
        e2e_ev[0].record(stream)
        plan.load_fields(host_fields)  # host -> device copy of this step's fields
        e2e_ev[1].record(stream)
        plan.replay()
        e2e_ev[2].record(stream)
        r_ = plan.result()
        host_series.copy_(plan.outputs, non_blocking=True)
        host_F.copy_(r_["Fsourceterm"], non_blocking=True)
        host_M2.copy_(r_["FsourcetermM2"], non_blocking=True)
        e2e_ev[3].record(stream)
        torch.cuda.synchronize()
        if it > 0:
            e_ms.append(e2e_ev[0].elapsed_time(e2e_ev[3]))
            e_parts.append([e2e_ev[i].elapsed_time(e2e_ev[i + 1]) for i in range(3)])
    clk_e2e.__exit__(None, None, None)
    e2e_ms = float(np.mean(e_ms))
    d2h = host_series.numel() * 8 + host_F.numel() * 16 + host_M2.numel() * 8

    # propagation kernel alone: launch duration for the roofline
    kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    kms = []
    for _ in range(2):
        l2_flush(flush)
        plan.launch(_events=kev)
        torch.cuda.synchronize()
        kms.append(kev[0].elapsed_time(kev[1]))
    k_ms = float(np.mean(kms))
    peak = ctypes_peak(lib, 0 if precision == "fp64" else 1)

    from mma_gb300 import autotune

    out = dict(value=value, ms_per_step=ms_step, S=S, n_inst=n_inst, kernel_ms=k_ms, peak=peak,
               cta_threads=int(grids.c64_threads[0]), m32=int(grids.m32[0]), autotune=autotune.last_report(),
               dft=autotune.dft_choice(S),
               clocks=clk.summary(), e2e_ms=e2e_ms, e2e_ms_each=e_ms, e2e_clocks=clk_e2e.summary(),
               e2e_parts_ms=[float(np.median([p[i] for p in e_parts])) for i in range(3)],
               h2d=host_fields.numel() * 8, d2h=d2h,
               t=t, fields=fields_np, spectrum=res["Fsourceterm"], omega=res["omegagrid"],
               sourceterm=res["sourceterm"])
    return out


def form_errors(test, ref, omega0=OMEGA0):
    """Errors of a form against the FP64 form on the same batch (the FP64 form equals the
    oracle within 1e-8), on the plateau |F|^2 (H11-H41) and the dipole (sourceterm):

    * ``plateau_rel_err_batch``: ||a - b|| / ||b|| over every instance together, the error that
      reaches the far field (which sums the instances);
    * median / p90 / max over the instances whose plateau holds at least 1e-3 of the strongest
      instance's plateau energy; instances at the weak-field edge of a focus have no plateau
      (cutoff below H11) and their relative error is the ratio of two round-off levels, so it
      is reported apart (``plateau_rel_err_max_all``)."""
    import torch

    om = ref["omega"]
    sel = (om >= 11 * omega0) & (om <= 41 * omega0)
    a = test["spectrum"][:, sel].abs() ** 2
    b = ref["spectrum"][:, sel].abs() ** 2
    nb = torch.linalg.norm(b, dim=1)
    pl = torch.linalg.norm(a - b, dim=1) / nb
    sig = nb >= 1e-3 * nb.max()
    ps = pl[sig]
    st = (torch.linalg.norm(test["sourceterm"] - ref["sourceterm"], dim=1) /
          torch.linalg.norm(ref["sourceterm"], dim=1))
    return {"plateau_rel_err_batch": float(torch.linalg.norm(a - b) / torch.linalg.norm(b)),
            "plateau_rel_err_median": float(ps.median()), "plateau_rel_err_p90": float(torch.quantile(ps, 0.9)),
            "plateau_rel_err_max": float(ps.max()), "plateau_instances": int(sig.sum()),
            "plateau_rel_err_max_all": float(pl.max()),
            "dipole_rel_l2_max": float(st.max()), "dipole_rel_l2_median": float(st.median())}


def ctypes_peak(lib, precision):
    import ctypes

    lib.mma_probe_fma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.mma_probe_fma_peak.restype = ctypes.c_int
    v = ctypes.c_double()
    rc = lib.mma_probe_fma_peak(precision, ctypes.byref(v))
    return v.value if rc == 0 else None


def load_traffic(name):
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except ValueError:
            return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-hankel", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the config-2 (uneven batch) and config-4 (adjoint) sub-lines of the default run")
    ap.add_argument("--fd-samples", type=int, default=None,
                    help="finite-difference samples per instance of the adjoint check (config 4: 32)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="config1")
    ap.add_argument("--ff-tol", type=float, default=1e-9,
                    help="series truncation bound of the fast far field (sets its number of terms)")
    ap.add_argument("--stage1", choices=("cuda", "tc"), default="cuda",
                    help="stage 1 of the fast far field: CUDA cores (default) or TF32 tensor cores")
    ap.add_argument("--forms", choices=["all", "both", "fp64", "c64", "df64"], default="all",
                    help="all: FP64, complex64 and float-float; both: FP64 and complex64")
    ap.add_argument("--c64-threads", default="auto",
                    help="CTA size of the complex64 kernel: auto (the autotuner) or 256, 512, 1024")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        t, fields = focus_fields()
        cores = os.cpu_count() or 1
        for _ in range(args.warmup):
            cpu_baseline(t, fields[:1], 1, cores=1)
        vals = []
        for _ in range(args.steps):
            vals.append(cpu_baseline(t, fields, cores, cores=cores))
        v = float(np.mean([x["value"] for x in vals]))
        line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "site-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "config1 TDSE batch sample on host cores (64r x 32z Gaussian focus, "
                                       "8001 sites, 4412 steps per instance)"},
                "cpu_baseline": {**vals[-1], "value": v},
                "e2e": {"value": v, "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    if args.workload in ("config0", "config2", "config3", "config4", "analysis", "small_wide", "small_adjoint",
                         "small_ff"):
        import torch

        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
        torch.cuda.set_device(dev)
        fn = {"config0": run_config0, "config2": run_config2, "config3": run_hankel, "small_ff": run_hankel,
              "config4": run_config4, "analysis": run_analysis, "small_wide": run_profile_case,
              "small_adjoint": run_profile_case}[args.workload]
        print(json.dumps({"workload": args.workload, "result": fn(args, dev)}))
        return
    # the headline form first, on a GPU not yet warmed by the other forms' runs
    rdf = run_ours(args, rank, world, "df64") if args.forms in ("all", "df64") else None
    r64 = run_ours(args, rank, world, "fp64") if args.forms in ("all", "both", "fp64") else None
    r = run_ours(args, rank, world, "c64") if args.forms in ("all", "both", "c64") else None
    if rank != 0:
        return
    if r is None or r64 is None or rdf is None:  # single-form run (profiling): a short line, no comparison
        one = rdf or r or r64
        print(json.dumps({"metric": METRIC, "value": one["value"], "unit": "site-steps/s", "forms": args.forms,
                          "workload": args.workload, "ms_per_step": one["ms_per_step"],
                          "kernel_ms": one["kernel_ms"]}))
        return
    site_steps = rdf["n_inst"] * 8001.0 * rdf["S"]
    err_df = form_errors(rdf, r64)
    err_c64 = form_errors(r, r64)
    # headline: the float-float form, the fastest form that meets the stated plateau error
    achieved = FLOPS_PER_SITE_STEP * site_steps / (rdf["kernel_ms"] * 1e-3)
    peak = rdf["peak"]
    prof = load_traffic("tdse_df64_config1.json") or {}
    roof = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12 if peak else None, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None,
            "traffic": prof.get("dram_bytes_per_launch"),
            "peak_source": "measured live: FP32 FMA loop on every SM (mma_probe_fma_peak); MEASURED_PEAKS.json "
                           "has no FP32 or FP64 figure",
            "kernel": "propagate_df64_kernel",
            "frac_of_fp64_peak": achieved / r64["peak"] if r64.get("peak") else None,
            "flops_per_site_step": FLOPS_PER_SITE_STEP,
            "fp32_instructions_per_site_step": prof.get("thread_instructions_per_site_step"),
            # the binding resource of the double-word arithmetic, from the committed ncu capture of
            # the same kernel (small_df workload, profiles/tdse_df64_propagate_small.md)
            "fp32_pipe_active_frac_ncu": (prof.get("fp32_pipe_active_pct") or 0.0) / 100.0 or None,
            "note": "achieved counts the 72 algorithmic FP64-equivalent flop per site-step; the kernel carries "
                    "each in double-word FP32 arithmetic (about 10 FP32 instructions per operation), so its "
                    "ceiling is the FP32 pipe (fp32_pipe_active_frac_ncu: the share of cycles the pipe was busy "
                    "in the ncu capture), not this fraction"}
    a64 = FLOPS_PER_SITE_STEP * site_steps / (r64["kernel_ms"] * 1e-3)
    a_c64 = FLOPS_PER_SITE_STEP * site_steps / (r["kernel_ms"] * 1e-3)
    target = 1e-6
    forms = {
        "tdse_plain_fp64": {"site_steps_per_s": r64["value"], "ms_per_step": r64["ms_per_step"],
                            "kernel_ms": r64["kernel_ms"], "roofline_frac_of_fp64_peak": a64 / r64["peak"],
                            "fp64_peak_tflops": r64["peak"] / 1e12, "e2e_site_steps_per_s":
                                world * site_steps / (r64["e2e_ms"] * 1e-3)},
        "tdse_float_float": {"site_steps_per_s": rdf["value"], "ms_per_step": rdf["ms_per_step"],
                             "kernel_ms": rdf["kernel_ms"], "speedup_vs_plain": rdf["value"] / r64["value"],
                             "algorithmic_tflops": achieved / 1e12,
                             "e2e_site_steps_per_s": world * site_steps / (rdf["e2e_ms"] * 1e-3),
                             "e2e_ms_each": rdf["e2e_ms_each"], "e2e_clocks": rdf["e2e_clocks"],
                             "e2e_parts_ms": {"fields_in": rdf["e2e_parts_ms"][0], "batch": rdf["e2e_parts_ms"][1],
                                              "results_out": rdf["e2e_parts_ms"][2],
                                              "d2h_gb_per_s": rdf["d2h"] / (rdf["e2e_parts_ms"][2] * 1e-3) / 1e9
                                              if rdf["e2e_parts_ms"][2] > 0 else None},
                             "error_vs_fp64": err_df,
                             "meets_plateau_target": err_df["plateau_rel_err_max"] <= target},
        "tdse_chosen_c64": {"site_steps_per_s": r["value"], "ms_per_step": r["ms_per_step"],
                            "kernel_ms": r["kernel_ms"], "speedup_vs_plain": r["value"] / r64["value"],
                            "algorithmic_tflops": a_c64 / 1e12,
                            "roofline_frac_of_fp32_peak": a_c64 / r["peak"] if r["peak"] else None,
                            "cta_threads": r["cta_threads"], "sites_per_thread": r["m32"],
                            "autotune_seconds_per_probe_batch": r["autotune"],
                            "error_vs_fp64": err_c64,
                            "meets_plateau_target": err_c64["plateau_rel_err_max"] <= target},
        "plateau_target": "|F|^2 over H11-H41 within %g relative of the FP64 form (which equals the oracle "
                          "within 1e-8)" % target,
        "spectrum_dft": dict(rdf["dft"], series_length=rdf["S"]),
    }
    line = {"metric": METRIC, "value": rdf["value"], "unit": "site-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rdf["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "df64 (float-float: FP32 pairs, about 48-bit significands; FP64 ground state and tables)",
            "data": "synthetic",
            "config": {"workload": "%s: %d TDSE instances (%d r x %d z Gaussian focus), 8001 sites, "
                                   "%d steps; headline form = float-float propagation (meets the 1e-6 plateau "
                                   "error); FP64 and complex64 under forms"
                                   % (args.workload, rdf["n_inst"], WORKLOADS[args.workload][0],
                                      WORKLOADS[args.workload][1], rdf["S"]),
                       "instances": rdf["n_inst"], "sites": 8001, "steps_per_instance": rdf["S"],
                       "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "forms": forms, "roofline": roof, "clocks": rdf["clocks"],
            "e2e": {"value": world * site_steps / (rdf["e2e_ms"] * 1e-3), "unit": "site-steps/s",
                    "h2d_bytes_per_step": rdf["h2d"], "d2h_bytes_per_step": rdf["d2h"]},
            "gpu_launches": GPU_LAUNCHES_PER_STEP * args.steps}
    if not args.no_hankel:
        import torch

        line["hankel"] = run_hankel(args, torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0))))
    if not args.no_extra and args.workload == "config1":
        import torch

        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
        # the uneven batch (config 2: 4096 instances, one launch per form) and the adjoint
        # (config 4: 256 instances, central finite differences at 4 samples per instance here;
        # `--workload config4` checks 32)
        line["config0"] = run_config0(args, dev)
        line["config2"] = run_config2(args, dev)
        if args.fd_samples is None:
            args.fd_samples = 4
        line["config4"] = run_config4(args, dev)
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(r["t"], r["fields"], 4 * (os.cpu_count() or 1))
        if not args.no_hankel:
            line["hankel"]["cpu_baseline"] = hankel_cpu_baseline()
    print(json.dumps(line))


if __name__ == "__main__":
    main()
