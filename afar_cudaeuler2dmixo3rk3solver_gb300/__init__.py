"""GB300-native AFAR per-stage residual + SSP-RK3 update (2-D compressible Euler, unstructured FV).

The compute path is libafar.so (csrc/: sm_103a CUDA kernels + C++ host precompute) behind the C ABI
in include/afar.h; this package is its Python host mirror (ctypes) plus the synthetic mesh
generators used by the tests and the benchmark.
"""
from . import mesh  # noqa: F401
from ._ffi import AfarError, lib  # noqa: F401
from .solver import (Batch, CaseConfig, CudaSolver, HostFields, Server, face_gauss_quadrature,  # noqa: F401
                     gauss_quadrature, precompute)

__all__ = ["Batch", "Server", "mesh", "lib", "AfarError", "CaseConfig", "CudaSolver", "HostFields", "precompute", "gauss_quadrature", "face_gauss_quadrature"]
