"""GB300-native engine for Tay's grid-structure simulation step.

The engine is native code (tay_gb300/libtay_gb300.so: CUDA kernels for sm_103a behind
the Tay C API in include/tay.h).  This package holds the build script, a ctypes mirror
of the C API (api), the host-side model descriptions (models) and seeded workloads
(workloads).
"""
from . import api, models, workloads  # noqa: F401
