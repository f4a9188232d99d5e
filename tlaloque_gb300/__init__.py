"""tlaloque_gb300: tlaloque's hydrodynamic time step on one GB300.

The product is libtlq.so (CUDA kernels for sm_103a behind the C ABI in
include/tlq.h); this package holds its sources (csrc/), its build
(build.py), the ctypes binding (tlq.py), the problem set-ups (problems.py)
and the analysis tools of the reference's test harness (analysis.py).
"""
from .tlq import Config, Context, TlqError, Wind, load_library  # noqa: F401

__all__ = ["Config", "Context", "TlqError", "Wind", "load_library"]
