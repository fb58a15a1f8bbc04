"""gpu_dsm_gb300 — GB300-native Discrete Slip-Link Model (DSM) kinetic Monte Carlo.

Python binding (ctypes) of the native library ``libgpudsm.so`` whose C ABI is
declared in ``include/dsm.h``.  The compute path is the hand-written sm_103a
CUDA of ``csrc/dsm_kernels.cu``; this module only moves host arrays in the
reference layout (ktaletsk/gpu_dsm common/chain.h:37-53) and calls the C ABI.
There is no CPU fallback: if the native library is missing, importing the
simulator raises.
"""
from .api import (  # noqa: F401
    HEAD_DTYPE,
    DSMError,
    Ensemble,
    Server,
    StressPlus,
    advance_batch,
    lib_path,
    load_library,
    gex_tables,
    make_params,
    pcd,
)

__all__ = ["HEAD_DTYPE", "DSMError", "Ensemble", "Server", "StressPlus", "advance_batch", "lib_path", "load_library", "make_params", "pcd", "gex_tables"]
