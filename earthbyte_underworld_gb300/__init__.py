"""GB300-native particle-in-cell Stokes hot path for Underworld 1.x models.

The compute lives in libuwgpu.so (CUDA C++ for sm_103a, C ABI in include/uwgpu.h); this package
holds its sources (csrc/), the in-tree build recipe (build.py), the ctypes binding (uwgpu.py),
the seeded workload generators (workloads.py) and the C host shim (host/).
"""
from . import build  # noqa: F401

__all__ = ["build", "uwgpu", "workloads"]
