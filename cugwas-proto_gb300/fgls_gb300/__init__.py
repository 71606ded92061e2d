"""GB300-native FGLS association engine (drop-in for the reference's
fgls_chol / fgls_eigen / fgls_chol_gpu).  The compute is the CUDA library
libfgls_gb300.so (built in-tree by ``fgls_gb300.build``); this package is its
Python mirror and the synthetic-data generator."""
from .engine import (Batch, Engine, FGLSError, fgls_chol, fgls_chol_gpu, fgls_eigen,  # noqa: F401
                     launch_count, lib, EXPORTS, LIB_PATH, DRIVER_PATH)

__all__ = ["Batch", "Engine", "FGLSError", "fgls_chol", "fgls_chol_gpu", "fgls_eigen", "launch_count", "lib",
           "EXPORTS", "LIB_PATH", "DRIVER_PATH"]
