"""GB300-native batched LU factor-and-solve behind MAGMA's batched C API.

The compute path is libmagma_lu.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/magma_lu.h).  This package is the Python host side: a
ctypes binding (`lib`), tensor-level wrappers (`batched`) and seeded input
generators (`testing`).
"""
from . import lib  # noqa: F401
from .batched import (Queue, VBatch, colmajor, dsgesv_batched, dsgesv_workspace_bytes,  # noqa: F401
                      from_colmajor, gesv_batched, gesv_vbatched, getrf_batched, getrs_batched,
                      ptr_array)

__all__ = ["lib", "Queue", "colmajor", "from_colmajor", "ptr_array", "getrf_batched",
           "getrs_batched", "gesv_batched", "dsgesv_batched", "dsgesv_workspace_bytes",
           "VBatch", "gesv_vbatched"]
