"""GB300-native implementation of MOM5's tracer-advection and split-explicit
barotropic path, behind the C ABI in include/mom5gpu.h.

Submodules:
  build    -- nvcc recipe for libmom5gpu.so (sm_103a)
  capi     -- ctypes binding of the C ABI (no fallback path)
  grid     -- seeded synthetic domains for the benchmark configurations
  harness  -- loads a synthetic domain into the library
"""
__all__ = ["build", "capi", "grid", "harness"]
