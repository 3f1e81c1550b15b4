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
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


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


def run_ours(args, rank, world, precision):
    import torch

    from mma_gb300 import load
    from mma_gb300.tdse_batch import TDSEGrids, run_batch

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    lib = load()
    t, fields_np = focus_fields()
    dtf = t[1] - t[0]
    tmax = t[-1] - t[0]
    n_inst = fields_np.shape[0]
    fields = torch.tensor(fields_np, device=dev)
    grids = TDSEGrids([dict(num_r=8000, dx=0.1, trg_a=A_CONFIG)], dt=dtf, c64=(precision == "c64"))
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    stream = torch.cuda.current_stream()

    def step():
        return run_batch(grids, fields, dt_field=dtf, tmax=tmax, precision=precision)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    S = int(step()["S"][0])
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
    ms_step = float(np.mean(ms))
    if world > 1:
        tt = torch.tensor([ms_step], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(tt.item())
    site_steps = float(n_inst) * sites * S
    value = world * site_steps / (ms_step * 1e-3)

    # propagation kernel alone: launch duration for the roofline
    kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    kms = []
    for _ in range(2):
        l2_flush(flush)
        r = run_batch(grids, fields, dt_field=dtf, tmax=tmax, spectra=False, _events=kev, precision=precision)
        torch.cuda.synchronize()
        kms.append(kev[0].elapsed_time(kev[1]))
    k_ms = float(np.mean(kms))
    peak = ctypes_peak(lib, 0 if precision == "fp64" else 1)

    # end to end through the public API: host (pinned) fields in, host spectra out
    host_fields = torch.tensor(fields_np).pin_memory()
    host_out = torch.empty((n_inst, S // 2 + 1), dtype=torch.complex128).pin_memory()
    e2e_ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    e_ms = []
    for _ in range(max(1, min(args.steps, 2))):
        l2_flush(flush)
        e2e_ev[0].record(stream)
        f_dev = host_fields.to(dev, non_blocking=True)
        rr = run_batch(grids, f_dev, dt_field=dtf, tmax=tmax, precision=precision)
        host_out.copy_(rr["Fsourceterm"], non_blocking=True)
        e2e_ev[1].record(stream)
        torch.cuda.synchronize()
        e_ms.append(e2e_ev[0].elapsed_time(e2e_ev[1]))
    e2e_ms = float(np.mean(e_ms))

    out = dict(value=value, ms_per_step=ms_step, S=S, n_inst=n_inst, kernel_ms=k_ms, peak=peak,
               clocks=clk.summary(), e2e_ms=e2e_ms, h2d=host_fields.numel() * 8, d2h=host_out.numel() * 16,
               t=t, fields=fields_np, spectrum=res["Fsourceterm"], omega=res["omegagrid"],
               sourceterm=res["sourceterm"])
    return out


def form_errors(test, ref, omega0=OMEGA0):
    """Errors of a form against the FP64 form on the same batch (the FP64 form equals the
    oracle within 1e-8): worst-instance plateau |F|^2 (H11-H41) and dipole relative L2."""
    import torch

    om = ref["omega"]
    sel = (om >= 11 * omega0) & (om <= 41 * omega0)
    a = test["spectrum"][:, sel].abs() ** 2
    b = ref["spectrum"][:, sel].abs() ** 2
    pl = (torch.linalg.norm(a - b, dim=1) / torch.linalg.norm(b, dim=1))
    st = (torch.linalg.norm(test["sourceterm"] - ref["sourceterm"], dim=1) /
          torch.linalg.norm(ref["sourceterm"], dim=1))
    return {"plateau_rel_err_max": float(pl.max()), "plateau_rel_err_median": float(pl.median()),
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
    r64 = run_ours(args, rank, world, "fp64")
    r = run_ours(args, rank, world, "c64")
    if rank != 0:
        return
    errs = form_errors(r, r64)
    site_steps = r["n_inst"] * 8001.0 * r["S"]
    achieved = FLOPS_PER_SITE_STEP * site_steps / (r["kernel_ms"] * 1e-3)
    peak = r["peak"]
    prof = load_traffic("tdse_c64_config1.json") or {}
    roof = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12 if peak else None, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None,
            "traffic": prof.get("dram_bytes_per_launch"),
            "peak_source": "measured live: FP32 FMA loop on every SM (mma_probe_fma_peak)",
            "kernel": "propagate_c64_kernel<32>", "flops_per_site_step": FLOPS_PER_SITE_STEP}
    a64 = FLOPS_PER_SITE_STEP * site_steps / (r64["kernel_ms"] * 1e-3)
    forms = {
        "tdse_plain_fp64": {"site_steps_per_s": r64["value"], "ms_per_step": r64["ms_per_step"],
                            "kernel_ms": r64["kernel_ms"], "roofline_frac_of_fp64_peak": a64 / r64["peak"],
                            "fp64_peak_tflops": r64["peak"] / 1e12, "e2e_site_steps_per_s":
                                world * site_steps / (r64["e2e_ms"] * 1e-3)},
        "tdse_chosen_c64": {"site_steps_per_s": r["value"], "ms_per_step": r["ms_per_step"],
                            "kernel_ms": r["kernel_ms"], "speedup_vs_plain": r["value"] / r64["value"],
                            "error_vs_fp64": errs},
    }
    line = {"metric": METRIC, "value": r["value"], "unit": "site-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 (fp32 propagation, fp64 factorisation/accumulation)",
            "data": "synthetic",
            "config": {"workload": "config1: 2048 TDSE instances (64 r x 32 z Gaussian focus), 8001 sites, "
                                   "%d steps; chosen form = complex64 propagation" % r["S"],
                       "instances": r["n_inst"], "sites": 8001, "steps_per_instance": r["S"],
                       "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "forms": forms, "roofline": roof, "clocks": r["clocks"],
            "e2e": {"value": world * site_steps / (r["e2e_ms"] * 1e-3), "unit": "site-steps/s",
                    "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": 3 * args.steps}
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(r["t"], r["fields"], os.cpu_count() or 1)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
