"""ctypes wrapper of liblapack_cpu.so (lapack_cpu.c): the reference's CPU path
for batched solves -- LAPACK dgesv per matrix under OpenMP with one BLAS thread
(testing/testing_zgesv_batched.cpp:160-176) -- against the LAPACK bundled with
scipy.  Benchmark and test infrastructure only.

`available()` is False when scipy or its bundled OpenBLAS is not installed; the
benchmark then times the oracle port instead and says so.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "lapack_cpu.c"
LIB = HERE / "liblapack_cpu.so"
_lock = threading.Lock()
_lib = None
_err = None


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(SRC), "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"lapack_cpu build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def lapack_path() -> str | None:
    """The OpenBLAS library scipy ships (scipy.libs/libscipy_openblas*.so), or None."""
    try:
        import scipy
    except ImportError:
        return None
    base = Path(scipy.__file__).resolve().parent.parent
    cands = sorted(glob.glob(str(base / "scipy.libs" / "libscipy_openblas*.so*")))
    return cands[0] if cands else None


def load():
    global _lib, _err
    with _lock:
        if _lib is None and _err is None:
            path = lapack_path()
            if path is None:
                _err = "scipy's bundled OpenBLAS not found"
                return None
            build()
            lib = C.CDLL(str(LIB))
            lib.lapack_open.argtypes = [C.c_char_p]
            if lib.lapack_open(path.encode()) != 0:
                _err = f"could not load LAPACK symbols from {os.path.basename(path)}"
                return None
            _lib = lib
        return _lib


def available() -> bool:
    return load() is not None


def unavailable_reason() -> str | None:
    load()
    return _err


def library_name() -> str:
    p = lapack_path()
    return os.path.basename(p) if p else "none"


def max_threads() -> int:
    lib = load()
    return int(lib.lapack_max_threads()) if lib else os.cpu_count() or 1


def _ptrs(mats) -> np.ndarray:
    return np.array([m.ctypes.data for m in mats], dtype=np.uintp)


def _i32(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32))


def dgesv_list(As, Bs, nthreads=None) -> np.ndarray:
    """In place: As[k] (ncols, ld) column-major FP64, Bs[k] (nrhs, ldb).  Returns info."""
    lib = load()
    b = len(As)
    n = _i32([a.shape[0] for a in As])
    lda = _i32([a.shape[1] for a in As])
    nrhs = _i32([x.shape[0] for x in Bs])
    ldb = _i32([x.shape[1] for x in Bs])
    info = np.zeros(b, dtype=np.int32)
    pa, pb = _ptrs(As), _ptrs(Bs)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.lapack_dgesv_ptrs.argtypes = [C.c_int] + [C.c_void_p] * 7 + [C.c_int, C.c_int]
    lib.lapack_dgesv_ptrs(b, p(n), p(nrhs), p(pa), p(lda), p(pb), p(ldb), p(info),
                          int(n.max(initial=1)), int(nthreads or max_threads()))
    return info


def dgesv_batched(S, X, nthreads=None) -> np.ndarray:
    """(batch, n, ld) and (batch, nrhs, ldb) column-major batches, in place."""
    return dgesv_list(list(S), list(X), nthreads)


def dgesv_adjoint_list(As, Bs, Gs, GAs, nthreads=None) -> np.ndarray:
    """Forward solve (Bs := X), transposed solve (Gs := A^{-T} G) and GAs[k] = -GB X^T."""
    lib = load()
    b = len(As)
    n = _i32([a.shape[0] for a in As])
    lda = _i32([a.shape[1] for a in As])
    nrhs = _i32([x.shape[0] for x in Bs])
    ldb = _i32([x.shape[1] for x in Bs])
    info = np.zeros(b, dtype=np.int32)
    pa, pb, pg, pga = _ptrs(As), _ptrs(Bs), _ptrs(Gs), _ptrs(GAs)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.lapack_dgesv_adjoint_ptrs.argtypes = [C.c_int] + [C.c_void_p] * 9 + [C.c_int, C.c_int]
    lib.lapack_dgesv_adjoint_ptrs(b, p(n), p(nrhs), p(pa), p(lda), p(pb), p(ldb), p(pg), p(pga),
                                  p(info), int(n.max(initial=1)), int(nthreads or max_threads()))
    return info
