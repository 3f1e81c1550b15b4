"""Host logic of the far-field API without a GPU: the argument checks of FarFieldPlan and of the
stage-1 switch, and the library's process-wide far-field switches and block copy, which reject
bad arguments before any CUDA call."""
import ctypes

import numpy as np
import pytest
import torch

MMA_OK = 0


def test_far_field_plan_wants_a_device_source():
    from mma_gb300 import hankel as H

    S = torch.zeros(3, 4, 8, dtype=torch.complex64)  # a host tensor
    with pytest.raises(ValueError, match="device"):
        H.FarFieldPlan(np.arange(4.0), np.arange(8.0), np.arange(3.0), np.arange(2.0), S, 1.0)


def test_stage1_form_switch():
    from mma_gb300 import hankel as H

    with pytest.raises(ValueError):
        H.set_stage1_form("fp64")
    H.set_stage1_form("tc")  # the library's setter: no device needed
    H.set_stage1_form("cuda")


def test_library_far_field_switches_and_block_copy_arguments():
    from mma_gb300 import load

    lib = load()
    lib.mma_hankel_set_stage1.argtypes = [ctypes.c_int]
    lib.mma_hankel_set_stage1.restype = ctypes.c_int
    assert lib.mma_hankel_set_stage1(2) != MMA_OK  # only 0 (tensor cores) and 1 (CUDA cores)
    assert lib.mma_hankel_set_stage1(1) == MMA_OK
    lib.mma_hankel_test_ring_timeout.argtypes = [ctypes.c_int]
    lib.mma_hankel_test_ring_timeout.restype = ctypes.c_int
    assert lib.mma_hankel_test_ring_timeout(0) == MMA_OK
    lib.mma_hankel_copy_block.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                          ctypes.c_int64, ctypes.c_void_p]
    lib.mma_hankel_copy_block.restype = ctypes.c_int
    buf = (ctypes.c_char * 64)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    assert lib.mma_hankel_copy_block(None, p, 1, 16, 16, None) != MMA_OK  # no destination
    assert lib.mma_hankel_copy_block(p, p, 0, 16, 16, None) != MMA_OK  # no planes
    assert lib.mma_hankel_copy_block(p, p, 2, 8, 16, None) != MMA_OK  # block wider than the plane pitch
    assert lib.mma_hankel_copy_block(p, p, 2, 16, 0, None) != MMA_OK  # empty block


def test_series_cut_meets_the_plan_bound():
    """The cut-offs behind the fast far field's series length (host only): at the cut-off x for m
    terms, x^m / m! e^x stays within the plan's truncation bound, and 1e-5 above it exceeds it;
    the cut-offs grow with m, and m = n_terms reaches the plan's own x_max."""
    from math import exp, factorial

    from mma_gb300 import hankel as H

    lib = H._sig()
    lib.mma_hankel_series_cut.argtypes = [ctypes.POINTER(H.FastPlan), ctypes.c_int]
    lib.mma_hankel_series_cut.restype = ctypes.c_double
    omega0 = 0.057 / 2.4188843265857e-17
    z = np.ascontiguousarray(np.linspace(-5e-3, 5e-3, 256)[:-1])
    plan = H.FastPlan()
    assert lib.mma_hankel_fast_plan(z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(z), 1.0, 42 * omega0,
                                    200e-6, 5e-3, 1e-9, ctypes.byref(plan)) == MMA_OK
    d = plan.as_dict()
    M, tb = int(d["n_terms"]), float(d["trunc_bound"])
    x_max = 0.5 * float(d["sigma"]) * float(d["y_max"])

    def bound(x, m):
        return x ** m / factorial(m) * exp(x)

    cuts = {}
    for m in (M - 8, M - 4):
        x = lib.mma_hankel_series_cut(ctypes.byref(plan), m)
        assert 0.0 < x < x_max
        assert bound(x, m) <= tb * (1 + 1e-9)
        assert bound(x * (1 + 1e-5), m) > tb
        cuts[m] = x
    assert cuts[M - 8] < cuts[M - 4]
    assert abs(lib.mma_hankel_series_cut(ctypes.byref(plan), M) - x_max) <= 1e-6 * x_max
    assert lib.mma_hankel_series_cut(ctypes.byref(plan), 1) == -1.0


def test_truncated_series_reproduces_j0_within_the_bound():
    """The mathematics of the fast far field's series length, independently of the kernels: for
    config 3's plan, every plane's J0(lambda_k y) = sum_m v_k^m K_m(y), K_m = (sigma y / 2)^m J_m(y)
    / m!, truncated at the length the cut-offs pick for x = sigma y / 2 (MM - 8, MM - 4 or MM terms),
    stays within the plan's truncation bound, for y over (0, y_max]."""
    from math import factorial

    from scipy.special import jv

    from mma_gb300 import hankel as H

    lib = H._sig()
    lib.mma_hankel_series_cut.argtypes = [ctypes.POINTER(H.FastPlan), ctypes.c_int]
    lib.mma_hankel_series_cut.restype = ctypes.c_double
    omega0 = 0.057 / 2.4188843265857e-17
    z = np.ascontiguousarray(np.linspace(-5e-3, 5e-3, 256)[:-1])
    plan = H.FastPlan()
    assert lib.mma_hankel_fast_plan(z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(z), 1.0, 42 * omega0,
                                    200e-6, 5e-3, 1e-9, ctypes.byref(plan)) == MMA_OK
    d = plan.as_dict()
    M, tb, sigma, d_ref, y_max = int(d["n_terms"]), d["trunc_bound"], d["sigma"], d["d_ref"], d["y_max"]
    cut8 = lib.mma_hankel_series_cut(ctypes.byref(plan), M - 8)
    cut4 = lib.mma_hankel_series_cut(ctypes.byref(plan), M - 4)
    lam = d_ref / (1.0 - z)  # D_k = distance - z_k
    v = (1.0 - lam ** 2) / sigma
    assert np.all(np.abs(v) <= 1 + 1e-12)
    y = np.concatenate([np.linspace(1e-3, 1.0, 200), np.linspace(1.0, y_max, 2000)])
    x = 0.5 * sigma * y
    n_terms = np.where(x <= cut8, M - 8, np.where(x <= cut4, M - 4, M))
    assert (n_terms == M - 8).any() and (n_terms == M - 4).any() and (n_terms == M).any()
    K = np.stack([(0.5 * sigma * y) ** m / factorial(m) * jv(m, y) for m in range(M)])  # [m, y]
    for k in range(0, len(z), 17):
        terms = v[k] ** np.arange(M)[:, None] * K
        mask = np.arange(M)[:, None] < n_terms[None, :]
        series = (terms * mask).sum(axis=0)
        err = np.abs(series - jv(0, lam[k] * y))
        assert err.max() <= tb + 1e-13, (k, err.max(), tb)
