"""GB300-native microscopic-to-far-field path of the MMA high-harmonic model.

* ``mma_gb300.tdse``        -- drop-in host class for the TDSE C-ABI (``TDSE_DLL``)
* ``mma_gb300.structures``  -- ctypes records with the reference DLL's layout
* ``mma_gb300.tdse_batch``  -- batched TDSE on torch device tensors
* ``mma_gb300.hankel``      -- the Hankel_transform.py entry points on the GPU

All compute runs in libmma_gb300.so (hand-written CUDA for sm_103a).
"""
from ._lib import MMAUnavailable, lib_path, load  # noqa: F401

__all__ = ["load", "lib_path", "MMAUnavailable"]
