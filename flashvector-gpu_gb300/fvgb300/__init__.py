"""fvgb300 -- GB300-native (sm_103a) distance-scan path of FlashVector-GPU.

The compute lives in libfvgb300.so (hand-written CUDA behind a C ABI, see
include/fv_bridge.h); this package loads it and mirrors the reference's
host-side interface for the scan path.
"""
from . import _lib, datasets  # noqa: F401

__all__ = ["_lib", "datasets"]
__version__ = "0.1.0"
