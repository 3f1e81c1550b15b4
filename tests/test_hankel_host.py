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
