"""GB300-native DEM time step with the xdynamics DEM launcher API.

Modules:
  types      ctypes mirrors of the structs in include/xdem_c.h
  scenes     synthetic scenes in the reference layout
  build      in-tree build of libxdem_gb300.so (sm_103a)
  _lib       ctypes binding of the library (no fallback when it is missing)
  launchers  the reference-named launchers on device mirrors of host arrays
  sim        the scene handle (fused sorted-order step)
"""
from . import types  # noqa: F401

__all__ = ["types", "scenes", "build", "launchers", "sim"]
