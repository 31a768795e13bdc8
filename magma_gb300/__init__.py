"""GB300-native batched LU factor-and-solve behind MAGMA's batched C API.

The compute path is libmagma_lu.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/magma_lu.h).  This package is the Python host side: a
ctypes binding (`lib`), tensor-level wrappers (`batched`) and seeded input
generators (`testing`).
"""
from . import lib  # noqa: F401
from .batched import (Queue, VBatch, autotune_getrf_batched, autotune_vbatched, colmajor,  # noqa: F401
                      dsgesv_batched, dsposv_batched, getrf_batched_tuning, load_tuning, save_tuning,
                      set_getrf_batched_tuning,
                      dsgesv_adjoint_batched, dxgesv_adjoint_vbatched, dxgesv_vbatched,
                      dsgesv_workspace_bytes, from_colmajor, gesv_batched, gesv_vbatched,
                      getrf_batched, getrs_batched, ptr_array, set_vbatched_tuning,
                      vbatched_tuning)

__all__ = ["lib", "Queue", "colmajor", "from_colmajor", "ptr_array", "getrf_batched",
           "getrs_batched", "gesv_batched", "dsgesv_batched", "dsposv_batched", "dsgesv_workspace_bytes",
           "VBatch", "gesv_vbatched", "vbatched_tuning", "set_vbatched_tuning",
           "autotune_vbatched", "dxgesv_vbatched", "dsgesv_adjoint_batched",
           "dxgesv_adjoint_vbatched", "autotune_getrf_batched", "getrf_batched_tuning",
           "set_getrf_batched_tuning", "save_tuning", "load_tuning"]
