"""ctypes wrapper of liblu_oracle.so (lu_oracle.c).  Test infrastructure only.

Arrays follow LAPACK conventions: a batch of column-major matrices is a numpy
array of shape (batch, ncols, ld) with element [k, j, i] = A_k(i, j), the same
storage the GPU library uses.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "lu_oracle.c"
LIB = HERE / "liblu_oracle.so"
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> Path:
    """Compile lu_oracle.c with gcc (no FMA contraction, OpenMP over the batch)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = C.CDLL(str(LIB))
        return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def max_threads() -> int:
    return int(load().oracle_max_threads())


def _threads(nthreads):
    return max_threads() if nthreads is None else int(nthreads)


def _getrf(prefix, A, m=None, nthreads=None):
    """In-place LU of a (batch, ncols, ld) column-major batch. Returns (ipiv, info)."""
    lib = load()
    dt = np.float64 if prefix == "d" else np.float32
    assert A.dtype == dt and A.flags.c_contiguous and A.ndim == 3
    b, n, ld = A.shape
    m = ld if m is None else m
    mn = max(min(m, n), 1)
    ipiv = np.zeros((b, mn), dtype=np.int32)
    info = np.zeros((b,), dtype=np.int32)
    fn = getattr(lib, f"oracle_{prefix}getrf_batched")
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_long,
                   C.c_void_p, C.c_int, C.c_int]
    fn(m, n, _p(A), ld, n * ld, _p(ipiv), mn, _p(info), b, _threads(nthreads))
    return ipiv, info


def _getrs(prefix, LU, ipiv, B, trans=False, nthreads=None):
    lib = load()
    dt = np.float64 if prefix == "d" else np.float32
    assert LU.dtype == dt and B.dtype == dt and B.flags.c_contiguous
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    b, n, ld = LU.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    fn = getattr(lib, f"oracle_{prefix}getrs_batched")
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p,
                   C.c_long, C.c_void_p, C.c_int, C.c_long, C.c_int, C.c_int]
    fn(1 if trans else 0, n, nrhs, _p(LU), ld, n * ld, _p(ipiv), ipiv.shape[1], _p(B), ldb,
       nrhs * ldb, b, _threads(nthreads))
    return B


def _gesv(prefix, A, B, nthreads=None):
    lib = load()
    dt = np.float64 if prefix == "d" else np.float32
    assert A.dtype == dt and B.dtype == dt and A.flags.c_contiguous and B.flags.c_contiguous
    b, n, ld = A.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    ipiv = np.zeros((b, max(n, 1)), dtype=np.int32)
    info = np.zeros((b,), dtype=np.int32)
    fn = getattr(lib, f"oracle_{prefix}gesv_batched")
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_long,
                   C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_int, C.c_int]
    fn(n, nrhs, _p(A), ld, n * ld, _p(ipiv), ipiv.shape[1], _p(B), ldb, nrhs * ldb, _p(info), b,
       _threads(nthreads))
    return ipiv, info


def dgetrf_batched(A, m=None, nthreads=None):
    return _getrf("d", A, m, nthreads)


def sgetrf_batched(A, m=None, nthreads=None):
    return _getrf("s", A, m, nthreads)


def dgetrs_batched(LU, ipiv, B, trans=False, nthreads=None):
    return _getrs("d", LU, ipiv, B, trans, nthreads)


def sgetrs_batched(LU, ipiv, B, trans=False, nthreads=None):
    return _getrs("s", LU, ipiv, B, trans, nthreads)


def dgesv_batched(A, B, nthreads=None):
    return _gesv("d", A, B, nthreads)


def sgesv_batched(A, B, nthreads=None):
    return _gesv("s", A, B, nthreads)


def dgetrf(A2, m=None):
    """Single matrix, (ncols, ld) storage."""
    A = A2[None]
    ipiv, info = dgetrf_batched(A, m, nthreads=1)
    return ipiv[0], int(info[0])


def sgetrf(A2, m=None):
    A = A2[None]
    ipiv, info = sgetrf_batched(A, m, nthreads=1)
    return ipiv[0], int(info[0])


def dgetrs(LU2, ipiv1, B2, trans=False):
    dgetrs_batched(LU2[None], ipiv1[None], B2[None], trans, nthreads=1)
    return B2


def sgetrs(LU2, ipiv1, B2, trans=False):
    sgetrs_batched(LU2[None], ipiv1[None], B2[None], trans, nthreads=1)
    return B2


def dgesv_vbatched(ns, nrhss, As, Bs, nthreads=None):
    """Variable-size batch: lists of (n_k, ld_k) / (nrhs_k, ldb_k) column-major arrays,
    solved in place.  Returns (list of ipiv arrays, info array)."""
    lib = load()
    b = len(ns)
    offA = np.zeros(b, dtype=np.int64)
    offB = np.zeros(b, dtype=np.int64)
    offP = np.zeros(b, dtype=np.int64)
    lda = np.array([a.shape[1] for a in As], dtype=np.int32)
    ldb = np.array([x.shape[1] for x in Bs], dtype=np.int32)
    na = np.array(ns, dtype=np.int32)
    nr = np.array(nrhss, dtype=np.int32)
    offA[1:] = np.cumsum([a.size for a in As])[:-1]
    offB[1:] = np.cumsum([x.size for x in Bs])[:-1]
    offP[1:] = np.cumsum(na)[:-1]
    Aflat = np.concatenate([a.ravel() for a in As]).astype(np.float64)
    Bflat = np.concatenate([x.ravel() for x in Bs]).astype(np.float64)
    P = np.zeros(max(int(na.sum()), 1), dtype=np.int32)
    info = np.zeros(b, dtype=np.int32)
    fn = lib.oracle_dgesv_vbatched
    fn.argtypes = [C.c_void_p] * 11 + [C.c_int, C.c_int]
    fn(_p(na), _p(nr), _p(Aflat), _p(offA), _p(lda), _p(P), _p(offP), _p(Bflat), _p(offB),
       _p(ldb), _p(info), b, _threads(nthreads))
    for k in range(b):
        As[k][...] = Aflat[offA[k]:offA[k] + As[k].size].reshape(As[k].shape)
        Bs[k][...] = Bflat[offB[k]:offB[k] + Bs[k].size].reshape(Bs[k].shape)
    pivs = [P[offP[k]:offP[k] + ns[k]].copy() for k in range(b)]
    return pivs, info


def sgesv_vbatched(ns, nrhss, As, Bs):
    """FP32 variable-size batch, same conventions as dgesv_vbatched (oracle_sgetrf + oracle_sgetrs
    per matrix, the solve applied whatever info is)."""
    pivs, info = [], np.zeros(len(ns), dtype=np.int32)
    for k in range(len(ns)):
        p, info[k] = sgetrf(As[k], ns[k])
        if nrhss[k] > 0 and ns[k] > 0:
            sgetrs(As[k], p, Bs[k])
        pivs.append(p[:ns[k]].copy())
    return pivs, info


def dsgesv_batched(A, B, itermax=30, tol=0.0, fallback=True, nthreads=None):
    """Mixed-precision IR restatement (oracle_dsgesv).  A: (batch, n, ld) FP64
    storage, modified only for matrices that fall back; B: (batch, nrhs, ldb).
    Returns (X, ipiv, info, iters) with X of B's shape."""
    lib = load()
    assert A.dtype == np.float64 and B.dtype == np.float64
    b, n, ld = A.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    X = np.zeros_like(B)
    ipiv = np.zeros((b, max(n, 1)), dtype=np.int32)
    info = np.zeros((b,), dtype=np.int32)
    iters = np.zeros((b,), dtype=np.int32)
    fn = lib.oracle_dsgesv_batched
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_int, C.c_long,
                   C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p,
                   C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]
    fn(n, nrhs, _p(A), ld, n * ld, _p(B), ldb, nrhs * ldb, _p(X), ldb, nrhs * ldb, _p(ipiv),
       ipiv.shape[1], _p(info), _p(iters), itermax, float(tol), 1 if fallback else 0, b,
       _threads(nthreads))
    return X, ipiv, info, iters


def dsgesv_gmres_batched(A, B, itermax=30, tol=0.0, fallback=True, nthreads=None):
    """GMRES-based refinement restatement (oracle_dsgesv_gmres): as
    dsgesv_batched, each correction solved by FP32 GMRES preconditioned with the
    FP32 factors; iters counts inner iterations."""
    lib = load()
    assert A.dtype == np.float64 and B.dtype == np.float64
    b, n, ld = A.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    X = np.zeros_like(B)
    ipiv = np.zeros((b, max(n, 1)), dtype=np.int32)
    info = np.zeros((b,), dtype=np.int32)
    iters = np.zeros((b,), dtype=np.int32)
    fn = lib.oracle_dsgesv_gmres_batched
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_int, C.c_long,
                   C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p,
                   C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]
    fn(n, nrhs, _p(A), ld, n * ld, _p(B), ldb, nrhs * ldb, _p(X), ldb, nrhs * ldb, _p(ipiv),
       ipiv.shape[1], _p(info), _p(iters), itermax, float(tol), 1 if fallback else 0, b,
       _threads(nthreads))
    return X, ipiv, info, iters


def dsposv_batched(A, B, itermax=30, tol=0.0, fallback=True, nthreads=None):
    """Mixed-precision SPD refinement restatement (oracle_dsposv): FP32 Cholesky
    (lower), FP64 refinement, FP64 posv fallback.  Returns (X, info, iters)."""
    lib = load()
    assert A.dtype == np.float64 and B.dtype == np.float64
    b, n, ld = A.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    X = np.zeros_like(B)
    info = np.zeros((b,), dtype=np.int32)
    iters = np.zeros((b,), dtype=np.int32)
    fn = lib.oracle_dsposv_batched
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_int, C.c_long,
                   C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                   C.c_int, C.c_int, C.c_int]
    fn(n, nrhs, _p(A), ld, n * ld, _p(B), ldb, nrhs * ldb, _p(X), ldb, nrhs * ldb, _p(info),
       _p(iters), itermax, float(tol), 1 if fallback else 0, b, _threads(nthreads))
    return X, info, iters


def getrf_nopiv(A2, m=None):
    """LU without pivoting of one matrix, (ncols, ld) storage, in place.  Returns info."""
    lib = load()
    n, ld = A2.shape
    m = n if m is None else m
    fn = getattr(lib, "oracle_dgetrf_nopiv" if A2.dtype == np.float64 else "oracle_sgetrf_nopiv")
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int]
    assert A2.flags.c_contiguous
    return int(fn(m, n, _p(A2), ld))


def rbt_matrix(A2, u, v):
    """A <- U^T A V (oracle_rbt_matrix) on one (n, ld) FP64 storage array, in place."""
    lib = load()
    n, ld = A2.shape
    fn = lib.oracle_rbt_matrix
    fn.restype = None
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    fn(n, _p(A2), ld, _p(u), _p(v))
    return A2


def rbt_vectors(trans, B2, w, n):
    """B <- U^T B (trans) or V B on one (nrhs, ld) FP64 storage array, in place."""
    lib = load()
    nrhs, ld = B2.shape
    fn = lib.oracle_rbt_vectors
    fn.restype = None
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    w = np.ascontiguousarray(w, dtype=np.float64)
    fn(1 if trans else 0, n, nrhs, _p(w), _p(B2), ld)
    return B2


def potrf(A2):
    """Lower Cholesky of one (n, ld) storage array in place (oracle_?potrf).  Returns info."""
    lib = load()
    n, ld = A2.shape
    fn = getattr(lib, "oracle_dpotrf" if A2.dtype == np.float64 else "oracle_spotrf")
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int]
    return int(fn(n, _p(A2), ld))


def potrs(L2, B2):
    """Solve L L^T X = B in place (oracle_?potrs); L2 (n, ld), B2 (nrhs, ldb) storage."""
    lib = load()
    n, ld = L2.shape
    nrhs, ldb = B2.shape
    fn = getattr(lib, "oracle_dpotrs" if L2.dtype == np.float64 else "oracle_spotrs")
    fn.restype = None
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    fn(n, nrhs, _p(L2), ld, _p(B2), ldb)
    return B2


def getri(LU, ipiv):
    """Inverse from the LU factors, the GPU's order: Y = solve(L, U, I) column by column
    (getrs arithmetic, no interchanges), then column j of Y is column perm[j] of inv(A), perm
    the interchanges applied to 0..n-1.  LU: (n, ld) storage; returns (n, n) storage."""
    n = LU.shape[0]
    E = np.zeros((n, max(n, 1)), dtype=LU.dtype)
    E[np.arange(n), np.arange(n)] = 1
    ident = np.arange(1, n + 1, dtype=np.int32)
    (dgetrs if LU.dtype == np.float64 else sgetrs)(LU, ident, E)
    perm = np.arange(n)
    for k in range(n):
        p = int(ipiv[k]) - 1
        perm[k], perm[p] = perm[p], perm[k]
    Inv = np.empty((n, n), dtype=LU.dtype)
    Inv[perm] = E[:, :n]
    return Inv


def dsgesv_vbatched(As, Bs, itermax=30, tol=0.0, fallback=True):
    """Variable-size refinement: oracle_dsgesv per matrix.  As[k]: (n_k, ld_k) storage,
    Bs[k]: (nrhs_k, ldb_k).  Returns (Xs, ipivs, info, iters)."""
    Xs, pivs = [], []
    info = np.zeros(len(As), dtype=np.int32)
    iters = np.zeros(len(As), dtype=np.int32)
    for k, (A, B) in enumerate(zip(As, Bs)):
        X, p, inf, it = dsgesv_batched(A[None], B[None], itermax, tol, fallback, nthreads=1)
        Xs.append(X[0])
        pivs.append(p[0][:A.shape[0]].copy())
        info[k], iters[k] = inf[0], it[0]
    return Xs, pivs, info, iters


def dsgesv_adjoint(A, ipiv, X, G, iter_fwd, itermax=30, tol=0.0, fallback=True):
    """Adjoint of one refinement solve (oracle_dsgesv_adjoint).  A: (n, ld) storage as the
    forward call left it (overwritten on fallback), ipiv: (n,) int32, X and G: (nrhs, ld)
    storage.  Returns (GB, GA, info, iter) with GB like G and GA (n, n) storage."""
    lib = load()
    n, lda = A.shape
    nrhs, ldx = X.shape
    ldg = G.shape[1]
    assert A.flags.c_contiguous and A.dtype == np.float64
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    GB = np.zeros_like(G)
    GA = np.zeros((n, n), dtype=np.float64)
    it = np.zeros(1, dtype=np.int32)
    fn = lib.oracle_dsgesv_adjoint
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                   C.c_int, C.c_double, C.c_int, C.c_void_p]
    info = fn(n, nrhs, _p(A), lda, _p(ipiv), _p(np.ascontiguousarray(X)), ldx,
              _p(np.ascontiguousarray(G)), ldg, _p(GB), ldg, _p(GA), n, int(iter_fwd), itermax,
              float(tol), 1 if fallback else 0, _p(it))
    return GB, GA, int(info), int(it[0]), ipiv


def gesv_adjoint_batched(LU, ipiv, X, G, nthreads=None):
    """G <- A^{-T} G and returns GA = -G X^T (storage layout), the oracle's
    restatement of the adjoint.  LU (batch, n, ld), X and G (batch, nrhs, ld)."""
    lib = load()
    pre = "d" if LU.dtype == np.float64 else "s"
    b, n, ld = LU.shape
    nrhs, ldx = X.shape[1], X.shape[2]
    ldg = G.shape[2]
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    GA = np.zeros((b, n, n), dtype=LU.dtype)
    fn = getattr(lib, f"oracle_{pre}gesv_adjoint_batched")
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_long,
                   C.c_void_p, C.c_int, C.c_long, C.c_void_p, C.c_int, C.c_long, C.c_void_p,
                   C.c_int, C.c_long, C.c_int, C.c_int]
    fn(n, nrhs, _p(LU), ld, n * ld, _p(ipiv), ipiv.shape[1], _p(X), ldx, nrhs * ldx, _p(G), ldg,
       nrhs * ldg, _p(GA), n, n * n, b, _threads(nthreads))
    return GA
