"""Autotuners of the batched TDSE's launch shapes (the tuning step of the batching form).

Two knobs are tuned by measurement:

* the spectrum and interpolation DFTs' tiling, per transform length: the library's plan for a
  length (``mma_dft_plan_info``, made on first use) times its shared-memory kernel at 256 and at
  512 threads per row on a probe batch and keeps the faster; ``dft_choice(n)`` reports it;
* the CTA size of the complex64 kernel, per grid size, which also sets the partition depth of its
  tridiagonal solve (the sites per thread, M = n / CTA size, each thread's sequential sweep
  length between the CTA-wide scans): 256 threads x M sites, 512 x M/2
or 1024 x M/4 (where the grid fits the shared-memory kernel, n <= 8192 for 512 threads and
n <= 8192 with M = 8 for 1024).  More threads per instance hide more latency (the kernel is
latency-bound: three CTA-wide barriers per step, dependent sweeps); wider CTAs pay for wider
scans.  Which wins depends on the grid and the GPU, so it is measured:

  for each candidate CTA size, build the grid's tables for it, propagate a seeded synthetic
  batch (two instances per SM, a sin^2 pulse of `steps` steps) and time it with CUDA events
  on the launching stream (one warm-up, median of three); keep the fastest, but leave the
  256-thread default only for a gain of at least MARGIN (a short probe does not resolve
  smaller differences reliably).

Grids are bucketed by their sites per thread at 256 threads (8, 16, 24, 32: the buckets with
more than one kernel shape); the first grid of a bucket is timed and the choice holds for the
bucket.  Choices are cached per (device name, bucket, dt, precision) in memory and, when the
environment variable MMA_TUNE_CACHE names a file, in that JSON file across processes.
"""
import json
import os

import numpy as np
import torch

CANDIDATES = (256, 512, 1024)
DEFAULT = 256
MARGIN = 0.03
_MEM = {}
_LAST = {}  # key -> {cta_threads: seconds} of the last tuning run (for reports)


def bucket(n):
    """Sites per thread of an n-site grid at 256 threads, rounded up to a multiple of 8."""
    m = -(-int(n) // 256)
    return -(-m // 8) * 8


def _key(n, dt, precision, device):
    name = torch.cuda.get_device_name(torch.device(device))
    return "%s|m256=%d|dt=%.9g|%s" % (name, bucket(n), float(dt), precision)


def _load():
    path = os.environ.get("MMA_TUNE_CACHE")
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    _MEM[key] = value
    path = os.environ.get("MMA_TUNE_CACHE")
    if not path:
        return
    data = _load()
    data[key] = value
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidate_shapes(n):
    """[(cta_threads, m32)] the complex64 form has kernels for, for a grid of n sites."""
    from .tdse_batch import _sig

    lib = _sig()
    out = []
    for t in CANDIDATES:
        m32 = -(-int(n) // t)
        m32 = -(-m32 // 8) * 8
        if lib.mma_tdse_c64_shape_ok(t, m32):
            out.append((t, m32))
    return out


def time_c64_threads(n, dt, param, threads, device="cuda", steps=800, seed=0):
    """Seconds per batch (two instances per SM, `steps` steps) of the complex64 form with
    tables laid out for `threads` CTA threads."""
    from .tdse_batch import TDSEGrids, run_batch

    dev = torch.device(device)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    grids = TDSEGrids([param], dt, device=dev, c64=True, c64_threads=int(threads))
    if int(grids.c64_threads[0]) != int(threads):
        return None
    rng = np.random.default_rng(seed)
    n_inst = 2 * sms
    nf = max(steps - 2, 8)
    nf += nf % 2
    t = dt * np.arange(1, nf + 1)
    T = t[-1] + dt
    E0 = rng.uniform(0.03, 0.06, n_inst)
    fields = torch.tensor(np.stack([e * np.sin(np.pi * t / T) ** 2 * np.cos(0.057 * t) for e in E0]), device=dev)
    stream = torch.cuda.current_stream(dev)
    times = []
    for rep in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        run_batch(grids, fields, dt, precision="c64", spectra=False, _events=(e0, e1))
        torch.cuda.synchronize(dev)
        if rep:
            times.append(e0.elapsed_time(e1) * 1e-3)
    return float(np.median(times))


def choose_c64_threads(n, dt, param, device="cuda", retune=False):
    """The CTA size for the complex64 tables of a grid with n sites (measured once per size
    bucket, cached)."""
    shapes = candidate_shapes(n)
    if len(shapes) <= 1:
        return shapes[0][0] if shapes else 256
    key = _key(n, dt, "c64", device)
    if not retune:
        if key in _MEM:
            return int(_MEM[key]["cta_threads"])
        disk = _load()
        if key in disk:
            _MEM[key] = disk[key]
            return int(disk[key]["cta_threads"])
    timing = {}
    for t, _ in shapes:
        s = time_c64_threads(n, dt, param, t, device=device)
        if s is not None:
            timing[t] = s
    best = min(timing, key=timing.get)
    if DEFAULT in timing and timing[best] > (1.0 - MARGIN) * timing[DEFAULT]:
        best = DEFAULT
    _LAST[key] = timing
    _store(key, {"cta_threads": int(best), "seconds": {str(k): v for k, v in timing.items()}})
    return int(best)


def last_report():
    """{cache key: {cta_threads: seconds}} of the tuning runs made by this process."""
    return {k: dict(v) for k, v in _LAST.items()}


def dft_choice(n):
    """The tiling the DFT plan of a length-n real transform runs: {'fft_len': complex FFT
    length, 'bluestein': bool, 'cta_threads': 256 or 512 (one CTA per row, every pass in shared
    memory; 0 = one launch per pass through global memory for FFT lengths above 7168),
    'probe_ms': {threads: probe-batch ms}}.  Makes the plan on the current device if needed."""
    import ctypes

    from ._lib import load

    lib = load()
    lib.mma_dft_plan_info.argtypes = [ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3 + [
        ctypes.POINTER(ctypes.c_float)]
    lib.mma_dft_plan_info.restype = ctypes.c_int
    m, b, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ms = (ctypes.c_float * 2)()
    rc = lib.mma_dft_plan_info(int(n), ctypes.byref(m), ctypes.byref(b), ctypes.byref(t), ms)
    if rc != 0:
        raise RuntimeError("mma_dft_plan_info failed with status %d" % rc)
    return {"fft_len": m.value, "bluestein": bool(b.value), "cta_threads": t.value,
            "probe_ms": {256: float(ms[0]), 512: float(ms[1])}}
