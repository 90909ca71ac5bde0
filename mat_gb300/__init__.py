"""mat_gb300: GB300-native (sm_103a) dense-factorization hot path of Mat.

The compute lives in libmatgpu.so (hand-written CUDA behind a C ABI,
include/mat_gpu.h).  This package only binds it for Python callers, tests and
the benchmark.
"""
from ._lib import LIB_PATH, MatGpuError, load  # noqa: F401

__all__ = ["LIB_PATH", "MatGpuError", "load"]
