"""GB300-native batch ray traversal behind the RTGI wavefront tracer interface.

The product is the C-ABI library ``_lib/libgrt.so`` (declared in ``include/grt.h``) with
hand-written sm_103a kernels. This Python package is a thin host-side binding over that
C-ABI (ctypes), plus the seeded workload generators used by the tests and the benchmark.
"""
from . import _libs, workloads  # noqa: F401
