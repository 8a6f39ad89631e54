"""GB300-native (sm_103a) implementation of ProDM's MDR refactor / retrieve path.

The compute lives in the in-tree CUDA library libprodm_gb300.so (C ABI in
include/prodm_gb300.h); this package binds it with ctypes and uses torch only
for device memory and streams.
"""
from ._lib import ProdmError, load  # noqa: F401

__all__ = ["ProdmError", "load"]
