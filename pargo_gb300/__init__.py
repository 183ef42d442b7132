"""pargo_gb300 -- GB300-native focal raster operators with the PaRGO operator API.

Layout:
  include/pargo_gpu.h      the C ABI (one entry point per reference operator Run())
  pargo_gb300/csrc/        CUDA kernels (sm_103a) and the ABI implementation
  pargo_gb300/gpro/        gpro-compatible C++ host layer (Application, RasterLayer,
                           Neighborhood, RasterOperator, the four operators) + app mains
  pargo_gb300/abi.py       ctypes binding of the C ABI (Python callers, tests, bench)
  pargo_gb300/synth.py     seeded synthetic DEM workloads
"""
from . import _paths  # noqa: F401

__all__ = ["abi", "synth", "build"]
