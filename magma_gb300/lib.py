"""ctypes binding of libmagma_lu.so (the C ABI declared in include/magma_lu.h).

Loading fails loudly: there is no CPU fallback for any routine of this
package.  Function names and argument order are MAGMA's.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libmagma_lu.so"

_lock = threading.Lock()
_lib = None

c_int = C.c_int
c_ptr = C.c_void_p

# argtypes of each exported routine (all pointers as void*)
_PROTOS = {
    "magma_init": ([], c_int),
    "magma_finalize": ([], c_int),
    "magma_xerbla": ([C.c_char_p, c_int], None),
    "magma_queue_create_internal": ([c_int, c_ptr, C.c_char_p, C.c_char_p, c_int], None),
    "magma_queue_create_from_cuda_internal": (
        [c_int, c_ptr, c_ptr, c_ptr, c_ptr, C.c_char_p, C.c_char_p, c_int], None),
    "magma_queue_destroy_internal": ([c_ptr, C.c_char_p, C.c_char_p, c_int], None),
    "magma_queue_sync_internal": ([c_ptr, C.c_char_p, C.c_char_p, c_int], None),
    "magma_queue_get_device": ([c_ptr], c_int),
    "magma_queue_get_cuda_stream": ([c_ptr], c_ptr),
    "magma_malloc": ([c_ptr, C.c_size_t], c_int),
    "magma_malloc_pinned": ([c_ptr, C.c_size_t], c_int),
    "magma_free_internal": ([c_ptr, C.c_char_p, C.c_char_p, c_int], c_int),
    "magma_free_pinned_internal": ([c_ptr, C.c_char_p, C.c_char_p, c_int], c_int),
    "magma_setvector_internal": (
        [c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr, C.c_char_p, C.c_char_p, c_int], None),
    "magma_getvector_internal": (
        [c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr, C.c_char_p, C.c_char_p, c_int], None),
    "magma_dset_pointer": ([c_ptr, c_ptr, c_int, c_int, c_int, c_int, c_int, c_ptr], None),
    "magma_sset_pointer": ([c_ptr, c_ptr, c_int, c_int, c_int, c_int, c_int, c_ptr], None),
    "magma_iset_pointer": ([c_ptr, c_ptr, c_int, c_int, c_int, c_int, c_int, c_ptr], None),
}
for _p in "ds":
    _PROTOS[f"magma_{_p}getrf_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}getrf_batched_smallsq_noshfl"] = ([c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}getrs_batched"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}gesv_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}gesv_batched_small"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr, c_int, c_ptr], c_int)
for _p in "ds":
    _PROTOS[f"magma_{_p}getrf_vbatched"] = ([c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}getrs_vbatched"] = ([c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                            c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}gesv_vbatched"] = ([c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                           c_int, c_ptr], c_int)
_PROTOS["magma_dgetrf_vbatched_max_nocheck_work"] = (
    [c_ptr, c_ptr, c_int, c_int, c_int, c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
     C.POINTER(c_int), c_int, c_ptr], c_int)
_PROTOS["magma_dgesv_vbatched_max_nocheck_work"] = (
    [c_ptr, c_ptr, c_int, c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
     C.POINTER(c_int), c_int, c_ptr], c_int)
for _p in "ds":
    _PROTOS[f"magma_{_p}gesv_adjoint_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int,
                                                  c_ptr, c_int, c_ptr, c_int, c_int, c_ptr], c_int)
    _PROTOS[f"magmablas_{_p}ger_neg_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr,
                                                 c_int, c_int, c_ptr], c_int)
_PROTOS["magma_sgetrf_batched_tc"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_ptr,
                                       C.POINTER(C.c_size_t), c_int, c_ptr], c_int)
_PROTOS["magma_sgetrf_batched_tc_status"] = ([c_int, c_int, c_ptr, c_int, c_ptr], c_int)
_PROTOS["magma_dxgesv_batched_work"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int,
                                         c_ptr, c_int, c_ptr, c_ptr, c_int, C.c_double, c_int,
                                         c_ptr, C.POINTER(C.c_size_t), c_int, c_ptr], c_int)
_PROTOS["magma_dsgesv_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr, c_int,
                                   c_ptr, c_ptr, c_int, c_ptr], c_int)
_PROTOS["magma_dsgesv_batched_noalloc"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr,
                                           c_int, c_ptr, c_ptr, c_int, c_ptr], c_int)
_PROTOS["magma_dsgesv_batched_work"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr,
                                        c_int, c_ptr, c_ptr, c_int, C.c_double, c_int, c_ptr,
                                        C.POINTER(C.c_size_t), c_int, c_ptr], c_int)

for _p in "ds":
    _PROTOS[f"magma_{_p}getrf_vbatched_autotune"] = ([c_int, c_ptr, c_ptr, c_ptr], c_int)
    _PROTOS[f"magma_{_p}vbatched_tuning_get"] = ([c_ptr, c_ptr], c_int)
    _PROTOS[f"magma_{_p}vbatched_tuning_set"] = ([c_ptr, c_ptr], c_int)
_PROTOS["magma_dxgesv_vbatched_work"] = ([c_int, c_ptr, c_ptr, c_int, c_int, c_ptr, c_ptr, c_ptr,
                                          c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_int,
                                          C.c_double, c_int, c_ptr, C.POINTER(C.c_size_t), c_int,
                                          c_ptr], c_int)
_PROTOS["magma_dxgesv_adjoint_batched_work"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_ptr, c_int,
                                                 c_ptr, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr,
                                                 c_ptr, c_ptr, c_int, C.c_double, c_int, c_ptr,
                                                 C.c_size_t, c_int, c_ptr], c_int)
_PROTOS["magma_dxgesv_adjoint_vbatched_work"] = ([c_ptr, c_ptr, c_int, c_int, c_ptr, c_ptr, c_ptr,
                                                  c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                                  c_ptr, c_ptr, c_ptr, c_ptr, c_int, C.c_double,
                                                  c_int, c_ptr, C.c_size_t, c_int, c_ptr], c_int)
_PROTOS["magmablas_dger_neg_vbatched"] = ([c_ptr, c_ptr, c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                                           c_ptr, c_int, c_ptr], c_int)
for _p in "ds":
    _PROTOS[f"magma_{_p}getri_outofplace_batched"] = ([c_int, c_ptr, c_int, c_ptr, c_ptr, c_int,
                                                      c_ptr, c_int, c_ptr], c_int)
for _p in "ds":
    _PROTOS[f"magma_{_p}getrf_batched_strided"] = ([c_int, c_int, c_ptr, c_int, c_int, c_ptr, c_int,
                                                   c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}getrs_batched_strided"] = ([c_int, c_int, c_int, c_ptr, c_int, c_int, c_ptr,
                                                   c_int, c_ptr, c_int, c_int, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}gesv_batched_strided"] = ([c_int, c_int, c_ptr, c_int, c_int, c_ptr, c_int,
                                                  c_ptr, c_int, c_int, c_ptr, c_int, c_ptr], c_int)
for _p in "ds":
    _PROTOS[f"magma_{_p}getrf_nopiv_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr],
                                                 c_int)
    _PROTOS[f"magma_{_p}getrs_nopiv_batched"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_int,
                                                  c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}gesv_nopiv_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr,
                                                 c_int, c_ptr], c_int)
_PROTOS["magma_dgerbt_batched"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr, c_ptr,
                                    c_ptr, c_int, c_ptr], c_int)
_PROTOS["magmablas_dprbt_batched"] = ([c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, c_ptr], None)
_PROTOS["magmablas_dprbt_mtv_batched"] = ([c_int, c_int, c_ptr, c_ptr, c_int, c_int, c_ptr], None)
_PROTOS["magmablas_dprbt_mv_batched"] = ([c_int, c_int, c_ptr, c_ptr, c_int, c_int, c_ptr], None)
_PROTOS["magma_dgesv_rbt_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr],
                                      c_int)
for _p in "ds":
    _PROTOS[f"magma_{_p}potrf_batched"] = ([c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}potrs_batched"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_int,
                                            c_ptr], c_int)
    _PROTOS[f"magma_{_p}posv_batched"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr,
                                           c_int, c_ptr], c_int)
_PROTOS["magma_dxgesv_gmres_batched_work"] = ([c_int, c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_ptr,
                                               c_int, c_ptr, c_int, c_ptr, c_ptr, c_int, C.c_double,
                                               c_int, c_ptr, c_ptr, c_int, c_ptr], c_int)
_PROTOS["magma_dsposv_batched_work"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr, c_int,
                                         c_ptr, c_ptr, c_int, C.c_double, c_int, c_ptr, c_ptr,
                                         c_int, c_ptr], c_int)
_PROTOS["magma_dsposv_batched"] = ([c_int, c_int, c_int, c_ptr, c_int, c_ptr, c_int, c_ptr, c_int,
                                    c_ptr, c_ptr, c_int, c_ptr], c_int)
_PROTOS["magma_lu_launch_count"] = ([], C.c_longlong)
for _p in "ds":
    _PROTOS[f"magma_{_p}getrf_batched_autotune"] = ([c_int, c_int, c_ptr], c_int)
    _PROTOS[f"magma_{_p}getrf_batched_tuning_get"] = ([c_ptr, c_ptr, c_ptr], c_int)
    _PROTOS[f"magma_{_p}getrf_batched_tuning_set"] = ([c_ptr, c_ptr, c_ptr], c_int)
_PROTOS["magma_lu_tuning_save"] = ([C.c_char_p], c_int)
_PROTOS["magma_lu_tuning_load"] = ([C.c_char_p], c_int)
_PROTOS["magma_lu_fail_allocations"] = ([c_int], c_int)
_PROTOS["magma_sgetrf_batched_tc_wait_selftest"] = ([C.c_longlong, c_ptr, c_ptr], c_int)
_PROTOS["magma_lu_timing_start"] = ([c_int, c_int], c_int)
_PROTOS["magma_lu_timing_stop"] = ([C.POINTER(c_int), C.POINTER(c_int), C.POINTER(C.c_double)],
                                   c_int)

# kernel classes of magma_lu_timing_start
KERNEL_CLASSES = {"small_gesv": 1, "panel": 2, "swap_trsm": 3, "gemm": 4, "tc_update": 5,
                  "getrs": 6, "ir_residual": 7, "ir_solve": 8, "ir_init": 9, "vb_lu": 10,
                  "adj_ger": 11, "outer": 12}


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libmagma_lu.so (building it first if the CUDA toolkit is present)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if path is None:
            from . import build as _build
            if not _build.up_to_date():
                _build.build()
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build it with magma_gb300.build.build()")
        lib = C.CDLL(str(p))
        for name, (args, res) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


_lib_bc = None


def load_bounds_checked() -> C.CDLL:
    """The bounds-check build of the library (libmagma_lu_bc.so, built on first use
    with -DMLU_BOUNDS_CHECK): the same entry points, plus
    mlu_bounds_check_read(&first, &count, reset), the record of global accesses
    that fell outside their operand.  Test infrastructure; it loads beside the
    normal library without sharing state with it."""
    global _lib_bc
    with _lock:
        if _lib_bc is not None:
            return _lib_bc
        from . import build as _build
        p = _build.build_bounds_check()
        lib = C.CDLL(str(p))
        for name, (args, res) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        lib.mlu_bounds_check_read.argtypes = [C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong), C.c_int]
        lib.mlu_bounds_check_read.restype = C.c_int
        _lib_bc = lib
        return lib


def exported_names() -> list[str]:
    return sorted(_PROTOS)


MagmaNoTrans = 111
MagmaTrans = 112
MagmaConjTrans = 113
