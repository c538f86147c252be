"""scihpc_gb300 -- GB300 (sm_103a) implementation of SciHPC's two-phase projection step.

The product is the C-ABI shared library ``_lib/libscihpc_gb300.so`` (declarations in
``include/scihpc_gpu.h``).  ``scihpc_gb300.native`` is a thin ctypes binding of that ABI for
Python callers (tests, benchmarks); it raises if the library is missing rather than falling
back to any CPU path.
"""
from .native import (BC, Grid, Lib, LibraryNotBuilt, Poisson, ScihpcError, TwoPhase, UNet, Workspace, conv3x3,  # noqa: F401
                     conv3x3_wgrad, conv3x3x3, conv3x3x3_wgrad, lib)
