"""Tensor-level wrappers over the MAGMA batched LU C ABI.

Storage convention: a batch of column-major matrices is a CUDA tensor `S` of
shape (batch, ncols, ld) whose element S[k, j, i] is A_k(i, j) -- exactly the
memory MAGMA's dA_array[k][i + j*ldda] addresses.  `colmajor()` converts a
(batch, m, n) math-oriented tensor to that storage and `from_colmajor()` back.

Every routine enqueues on the current torch CUDA stream through a
magma_queue_t wrapping it, returns without synchronising, and raises
RuntimeError on a negative MAGMA return code.
"""
from __future__ import annotations

import ctypes as C
import threading

import torch

from . import lib as _L

_qlock = threading.Lock()
_queues: dict[tuple[int, int], "Queue"] = {}


class Queue:
    """magma_queue_t around an existing CUDA stream (magma_queue_create_from_cuda)."""

    def __init__(self, device: int, stream_handle: int):
        lib = _L.load()
        self._lib = lib
        h = C.c_void_p()
        lib.magma_queue_create_from_cuda_internal(device, C.c_void_p(stream_handle), None, None,
                                                  C.byref(h), b"Queue", b"batched.py", 0)
        if not h.value:
            raise RuntimeError("magma_queue_create_from_cuda failed")
        self.handle = h
        self.device = device
        self.stream_handle = stream_handle

    def sync(self):
        self._lib.magma_queue_sync_internal(self.handle, b"sync", b"batched.py", 0)

    def __del__(self):
        try:
            self._lib.magma_queue_destroy_internal(self.handle, b"del", b"batched.py", 0)
        except Exception:
            pass

    @staticmethod
    def current(device: torch.device | int | None = None) -> "Queue":
        if isinstance(device, int):
            dev = device
        elif device is not None and device.index is not None:
            dev = device.index
        else:
            dev = torch.cuda.current_device()
        s = torch.cuda.current_stream(dev).cuda_stream
        key = (dev, s)
        with _qlock:
            q = _queues.get(key)
            if q is None:
                q = Queue(dev, s)
                _queues[key] = q
            return q


def colmajor(A: torch.Tensor, ld: int | None = None) -> torch.Tensor:
    """(batch, m, n) -> column-major storage (batch, n, ld), ld >= m."""
    b, m, n = A.shape
    ld = m if ld is None else ld
    S = torch.zeros((b, n, ld), dtype=A.dtype, device=A.device)
    S[:, :, :m] = A.transpose(1, 2)
    return S


def from_colmajor(S: torch.Tensor, m: int) -> torch.Tensor:
    return S[:, :, :m].transpose(1, 2)


def ptr_array(S: torch.Tensor) -> torch.Tensor:
    """int64 device tensor holding the address of S[k] for every k (a T** array)."""
    step = S.stride(0) * S.element_size()
    return S.data_ptr() + torch.arange(S.shape[0], device=S.device, dtype=torch.int64) * step


def _prefix(t: torch.Tensor) -> str:
    if t.dtype == torch.float64:
        return "d"
    if t.dtype == torch.float32:
        return "s"
    raise TypeError(f"unsupported dtype {t.dtype}")


def _check(rc: int, name: str):
    if rc != 0:
        raise RuntimeError(f"{name} returned {rc}")


def _vp(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _check_storage(S: torch.Tensor, name: str):
    ok = S.is_cuda and S.dim() == 3 and (S.shape[2] <= 1 or S.stride(2) == 1) and \
        (S.shape[1] <= 1 or S.stride(1) == S.shape[2])
    if not ok:
        raise ValueError(f"{name} must be CUDA column-major storage (batch, ncols, ld), contiguous")


def getrf_batched(S: torch.Tensor, m: int | None = None, ipiv: torch.Tensor | None = None,
                  info: torch.Tensor | None = None, queue: Queue | None = None):
    """In-place LU of every matrix in S (magma_?getrf_batched). Returns (ipiv, info)."""
    _check_storage(S, "S")
    b, n, ld = S.shape
    m = ld if m is None else m
    mn = min(m, n)
    ipiv = torch.empty((b, max(mn, 1)), dtype=torch.int32, device=S.device) if ipiv is None else ipiv
    info = torch.empty((b,), dtype=torch.int32, device=S.device) if info is None else info
    q = queue or Queue.current(S.device)
    lib = _L.load()
    p = _prefix(S)
    # the pointer arrays must stay referenced until the call has enqueued its kernels
    dA = ptr_array(S)
    dP = ptr_array(ipiv)
    rc = getattr(lib, f"magma_{p}getrf_batched")(m, n, _vp(dA), ld, _vp(dP), _vp(info), b, q.handle)
    _check(rc, f"magma_{p}getrf_batched")
    return ipiv, info


def getrs_batched(LU: torch.Tensor, ipiv: torch.Tensor, B: torch.Tensor, trans: bool = False,
                  queue: Queue | None = None):
    """Solve op(A) X = B in place in B (magma_?getrs_batched)."""
    _check_storage(LU, "LU")
    _check_storage(B, "B")
    b, n, ld = LU.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    q = queue or Queue.current(LU.device)
    lib = _L.load()
    p = _prefix(LU)
    tr = _L.MagmaTrans if trans else _L.MagmaNoTrans
    dA, dP, dB = ptr_array(LU), ptr_array(ipiv), ptr_array(B)
    rc = getattr(lib, f"magma_{p}getrs_batched")(tr, n, nrhs, _vp(dA), ld, _vp(dP), _vp(dB), ldb,
                                                 b, q.handle)
    _check(rc, f"magma_{p}getrs_batched")
    return B


def gesv_batched(S: torch.Tensor, B: torch.Tensor, ipiv: torch.Tensor | None = None,
                 info: torch.Tensor | None = None, queue: Queue | None = None):
    """Factor S and solve in place (magma_?gesv_batched). Returns (ipiv, info)."""
    _check_storage(S, "S")
    _check_storage(B, "B")
    b, n, ld = S.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    ipiv = torch.empty((b, max(n, 1)), dtype=torch.int32, device=S.device) if ipiv is None else ipiv
    info = torch.empty((b,), dtype=torch.int32, device=S.device) if info is None else info
    q = queue or Queue.current(S.device)
    lib = _L.load()
    p = _prefix(S)
    dA, dP, dB = ptr_array(S), ptr_array(ipiv), ptr_array(B)
    rc = getattr(lib, f"magma_{p}gesv_batched")(n, nrhs, _vp(dA), ld, _vp(dP), _vp(dB), ldb,
                                                _vp(info), b, q.handle)
    _check(rc, f"magma_{p}gesv_batched")
    return ipiv, info


PRECISIONS = {"fp32": 900, "fp16": 905, "bf16": 930}


def dsgesv_batched(S: torch.Tensor, B: torch.Tensor, X: torch.Tensor | None = None,
                   itermax: int = 30, tol: float = 0.0, fallback: bool = True,
                   ipiv: torch.Tensor | None = None, info: torch.Tensor | None = None,
                   iters: torch.Tensor | None = None, work: torch.Tensor | None = None,
                   queue: Queue | None = None, precision: str = "fp32", solver: str = "ir"):
    """Batched FP32-factor / FP64-refinement solve (magma_dsgesv_batched_work).

    S and B are FP64 column-major storage and are left unchanged unless a
    matrix falls back to FP64 (then S holds its FP64 LU).  Returns
    (X, ipiv, info, iters).  `work` may be a preallocated uint8 CUDA tensor of
    at least dsgesv_workspace_bytes() bytes.  solver "gmres" solves each
    correction with GMRES preconditioned by the factors
    (magma_dxgesv_gmres_batched_work, Magma_REFINE_IRGMSTRS); iters then
    counts inner iterations."""
    _check_storage(S, "S")
    _check_storage(B, "B")
    if S.dtype != torch.float64 or B.dtype != torch.float64:
        raise TypeError("dsgesv_batched takes float64 inputs")
    b, n, ld = S.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    X = torch.empty_like(B) if X is None else X
    _check_storage(X, "X")
    ipiv = torch.empty((b, max(n, 1)), dtype=torch.int32, device=S.device) if ipiv is None else ipiv
    info = torch.empty((b,), dtype=torch.int32, device=S.device) if info is None else info
    iters = torch.empty((b,), dtype=torch.int32, device=S.device) if iters is None else iters
    q = queue or Queue.current(S.device)
    lib = _L.load()
    prec = PRECISIONS[precision]
    need = dsgesv_workspace_bytes(n, nrhs, b, precision, solver)
    if work is None or work.numel() < need:
        work = torch.empty((max(need, 1),), dtype=torch.uint8, device=S.device)
    lw = C.c_size_t(work.numel())
    dA, dP, dB, dX = ptr_array(S), ptr_array(ipiv), ptr_array(B), ptr_array(X)
    rc = lib.magma_dxgesv_gmres_batched_work(prec, SOLVERS[solver], n, nrhs, _vp(dA), ld, _vp(dP),
                                             _vp(dB), ldb, _vp(dX), X.shape[2], _vp(info),
                                             _vp(iters), itermax, float(tol), 1 if fallback else 0,
                                             _vp(work), C.byref(lw), b, q.handle)
    _check(rc, "magma_dxgesv_gmres_batched_work")
    return X, ipiv, info, iters


SOLVERS = {"ir": 920, "gmres": 922}


def dsposv_batched(S: torch.Tensor, B: torch.Tensor, X: torch.Tensor | None = None,
                   itermax: int = 30, tol: float = 0.0, fallback: bool = True,
                   queue: Queue | None = None):
    """Batched FP32-Cholesky / FP64-refinement SPD solve (magma_dsposv_batched_work,
    lower triangle).  S, B FP64 column-major storage; S is left unchanged unless a
    matrix falls back to FP64.  Returns (X, info, iters)."""
    _check_storage(S, "S")
    _check_storage(B, "B")
    b, n, ld = S.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    X = torch.empty_like(B) if X is None else X
    info = torch.empty((b,), dtype=torch.int32, device=S.device)
    iters = torch.empty((b,), dtype=torch.int32, device=S.device)
    q = queue or Queue.current(S.device)
    lib = _L.load()
    lw = C.c_size_t(0)
    rc = lib.magma_dsposv_batched_work(122, n, nrhs, None, max(ld, 1), None, max(ldb, 1), None,
                                       max(X.shape[2], 1), None, None, itermax, float(tol), 0,
                                       None, C.byref(lw), b, None)
    _check(rc, "magma_dsposv_batched_work(query)")
    work = torch.empty((max(int(lw.value), 1),), dtype=torch.uint8, device=S.device)
    lw = C.c_size_t(work.numel())
    dA, dB, dX = ptr_array(S), ptr_array(B), ptr_array(X)
    rc = lib.magma_dsposv_batched_work(122, n, nrhs, _vp(dA), ld, _vp(dB), ldb, _vp(dX),
                                       X.shape[2], _vp(info), _vp(iters), itermax, float(tol),
                                       1 if fallback else 0, _vp(work), C.byref(lw), b, q.handle)
    _check(rc, "magma_dsposv_batched_work")
    return X, info, iters


def dsgesv_workspace_bytes(n: int, nrhs: int, batch: int, precision: str = "fp32",
                           solver: str = "ir") -> int:
    lib = _L.load()
    lw = C.c_size_t(0)
    rc = lib.magma_dxgesv_gmres_batched_work(PRECISIONS[precision], SOLVERS[solver], n, nrhs, None,
                                             max(n, 1), None, None, max(n, 1), None, max(n, 1),
                                             None, None, 30, 0.0, 0, None, C.byref(lw), batch,
                                             None)
    _check(rc, "magma_dxgesv_gmres_batched_work(query)")
    return int(lw.value)


class VBatch:
    """A variable-size batch packed into one device buffer.

    mats: list of column-major storage tensors, matrix k of shape (ncols_k, ld_k)
    (that is, A_k^T in memory order).  The packed buffer holds them back to back
    (each start aligned to 64 bytes); `ptrs`, `ld`, `ncols` and `nrows` are the
    device arrays MAGMA's vbatched routines take."""

    def __init__(self, shapes, nrows, dtype, device):
        self.shapes = [tuple(s) for s in shapes]
        self.nrows = list(nrows)
        elsz = torch.empty((), dtype=dtype).element_size()
        align = 64 // elsz
        offs, o = [], 0
        for (nc, ld) in self.shapes:
            offs.append(o)
            o += ((nc * ld + align - 1) // align) * align
        self.offsets = offs
        self.buf = torch.zeros((max(o, 1),), dtype=dtype, device=device)
        base = self.buf.data_ptr()
        self.ptrs = torch.tensor([base + x * elsz for x in offs], dtype=torch.int64, device=device)
        self.ld = torch.tensor([ld for (_, ld) in self.shapes], dtype=torch.int32, device=device)
        self.ncols = torch.tensor([nc for (nc, _) in self.shapes], dtype=torch.int32, device=device)
        self.rows = torch.tensor(self.nrows, dtype=torch.int32, device=device)

    def view(self, k):
        nc, ld = self.shapes[k]
        o = self.offsets[k]
        return self.buf[o:o + nc * ld].view(nc, ld)

    def load(self, mats):
        for k, m in enumerate(mats):
            self.view(k).copy_(torch.as_tensor(m))
        return self


def gesv_vbatched(A: "VBatch", B: "VBatch", queue: Queue | None = None):
    """In-place factor and solve of a variable-size batch (magma_?gesv_vbatched).
    Returns (ipiv buffer, per-matrix ipiv offsets, info)."""
    b = len(A.shapes)
    lib = _L.load()
    p = _prefix(A.buf)
    n = A.ncols
    nrhs = B.ncols
    tot = sum(max(s[0], 1) for s in A.shapes)
    ipiv = torch.zeros((max(tot, 1),), dtype=torch.int32, device=A.buf.device)
    offs, o = [], 0
    for (nc, _) in A.shapes:
        offs.append(o)
        o += max(nc, 1)
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=A.buf.device) * 4
    info = torch.empty((b,), dtype=torch.int32, device=A.buf.device)
    q = queue or Queue.current(A.buf.device)
    rc = getattr(lib, f"magma_{p}gesv_vbatched")(_vp(n), _vp(nrhs), _vp(A.ptrs), _vp(A.ld), _vp(dP),
                                                 _vp(B.ptrs), _vp(B.ld), _vp(info), b, q.handle)
    _check(rc, f"magma_{p}gesv_vbatched")
    return ipiv, offs, info


def dxgesv_vbatched(A: "VBatch", B: "VBatch", X: "VBatch | None" = None, precision: str = "fp32",
                    itermax: int = 30, tol: float = 0.0, fallback: bool = True,
                    work: torch.Tensor | None = None, queue: Queue | None = None):
    """Mixed-precision refinement of a variable-size FP64 batch
    (magma_dxgesv_vbatched_work).  A is left intact except for matrices that fall back
    to the FP64 re-solve; B is read; X (allocated like B when None) receives the solutions.
    Returns (X, ipiv buffer, per-matrix ipiv offsets, info, iters, work); keep `work` (it
    holds the FP32 factors) for dxgesv_adjoint_vbatched."""
    if A.buf.dtype != torch.float64:
        raise TypeError("dxgesv_vbatched expects float64 batches")
    b = len(A.shapes)
    dev = A.buf.device
    lib = _L.load()
    if X is None:
        X = VBatch(B.shapes, B.nrows, torch.float64, dev)
    max_n = max([s[0] for s in A.shapes] + [0])
    max_r = max([s[0] for s in B.shapes] + [0])
    tot = sum(max(s[0], 1) for s in A.shapes)
    ipiv = torch.zeros((max(tot, 1),), dtype=torch.int32, device=dev)
    offs, o = [], 0
    for (nc, _) in A.shapes:
        offs.append(o)
        o += max(nc, 1)
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=dev) * 4
    info = torch.empty((b,), dtype=torch.int32, device=dev)
    iters = torch.empty((b,), dtype=torch.int32, device=dev)
    q = queue or Queue.current(dev)
    lw = C.c_size_t(0)
    args = (A.ncols, B.ncols)
    rc = lib.magma_dxgesv_vbatched_work(PRECISIONS[precision], _vp(args[0]), _vp(args[1]), max_n,
                                        max_r, None, None, None, None, None, None, None, None, None,
                                        itermax, float(tol), int(fallback), None, C.byref(lw), b,
                                        q.handle)
    _check(rc, "magma_dxgesv_vbatched_work(query)")
    if work is None or work.numel() < lw.value:
        work = torch.empty((max(lw.value, 1),), dtype=torch.uint8, device=dev)
    lw = C.c_size_t(work.numel())
    rc = lib.magma_dxgesv_vbatched_work(PRECISIONS[precision], _vp(A.ncols), _vp(B.ncols), max_n,
                                        max_r, _vp(A.ptrs), _vp(A.ld), _vp(dP), _vp(B.ptrs),
                                        _vp(B.ld), _vp(X.ptrs), _vp(X.ld), _vp(info), _vp(iters),
                                        itermax, float(tol), int(fallback), _vp(work),
                                        C.byref(lw), b, q.handle)
    _check(rc, "magma_dxgesv_vbatched_work")
    return X, ipiv, offs, info, iters, work


def dsgesv_adjoint_batched(S: torch.Tensor, ipiv: torch.Tensor, X: torch.Tensor, G: torch.Tensor,
                           iters_fwd: torch.Tensor, work: torch.Tensor, info: torch.Tensor,
                           itermax: int = 30, tol: float = 0.0, fallback: bool = True,
                           want_ga: bool = True, queue: Queue | None = None):
    """Adjoint of dsgesv_batched (magma_dxgesv_adjoint_batched_work): S, ipiv, X, iters_fwd,
    info and `work` as the forward call left them, G the upstream gradient of X (storage like
    X).  Returns (GB, GA, iters): GB = A^{-T} G (storage like G), GA = -GB X^T
    ((batch, n, n) storage) or None."""
    b, n, ld = S.shape
    nrhs = X.shape[1]
    GB = torch.empty_like(G)
    GA = torch.empty((b, n, n), dtype=torch.float64, device=S.device) if want_ga else None
    iters = torch.empty((b,), dtype=torch.int32, device=S.device)
    q = queue or Queue.current(S.device)
    dA, dP, dX, dG, dGB = ptr_array(S), ptr_array(ipiv), ptr_array(X), ptr_array(G), ptr_array(GB)
    dGA = ptr_array(GA) if want_ga else None
    rc = _L.load().magma_dxgesv_adjoint_batched_work(
        n, nrhs, _vp(dA), ld, _vp(dP), _vp(dX), X.shape[2], _vp(dG), G.shape[2], _vp(dGB),
        GB.shape[2], _vp(dGA) if want_ga else None, n, _vp(iters_fwd), _vp(info), _vp(iters),
        itermax, float(tol), int(fallback), _vp(work), work.numel(), b, q.handle)
    _check(rc, "magma_dxgesv_adjoint_batched_work")
    return GB, GA, iters


def dxgesv_adjoint_vbatched(A: "VBatch", ipiv: torch.Tensor, offs, X: "VBatch", G: "VBatch",
                            iters_fwd: torch.Tensor, info: torch.Tensor, work: torch.Tensor,
                            itermax: int = 30, tol: float = 0.0, fallback: bool = True,
                            want_ga: bool = True, queue: Queue | None = None):
    """Adjoint of dxgesv_vbatched (magma_dxgesv_adjoint_vbatched_work).  Returns
    (GB, GA, iters) with GB a VBatch like G and GA a VBatch of (n_k, n_k) matrices or None."""
    b = len(A.shapes)
    dev = A.buf.device
    GB = VBatch(G.shapes, G.nrows, torch.float64, dev)
    GA = VBatch([(s[0], s[0]) for s in A.shapes], [s[0] for s in A.shapes], torch.float64,
                dev) if want_ga else None
    iters = torch.empty((b,), dtype=torch.int32, device=dev)
    max_n = max([s[0] for s in A.shapes] + [0])
    max_r = max([s[0] for s in G.shapes] + [0])
    dP = ipiv.data_ptr() + torch.tensor(offs, dtype=torch.int64, device=dev) * 4
    q = queue or Queue.current(dev)
    rc = _L.load().magma_dxgesv_adjoint_vbatched_work(
        _vp(A.ncols), _vp(G.ncols), max_n, max_r, _vp(A.ptrs), _vp(A.ld), _vp(dP), _vp(X.ptrs),
        _vp(X.ld), _vp(G.ptrs), _vp(G.ld), _vp(GB.ptrs), _vp(GB.ld),
        _vp(GA.ptrs) if want_ga else None, _vp(GA.ld) if want_ga else None, _vp(iters_fwd),
        _vp(info), _vp(iters), itermax, float(tol), int(fallback), _vp(work), work.numel(), b,
        q.handle)
    _check(rc, "magma_dxgesv_adjoint_vbatched_work")
    return GB, GA, iters


# --------------------------------------------------------------------------
# tuning of the variable-size kernel

TUNE_BINS = ("<=16", "<=32", "<=64", "<=128", "<=256", "<=512", "<=1024", ">1024")
TILES = ("64x64", "32x64", "32x32")


def _tune_prefix(dtype: torch.dtype) -> str:
    if dtype == torch.float64:
        return "d"
    if dtype == torch.float32:
        return "s"
    raise TypeError(f"unsupported dtype {dtype}")


def _tune_dict(nb, tile) -> dict:
    return {b: {"nb": int(nb[i]), "tile": TILES[tile[i]]} for i, b in enumerate(TUNE_BINS)}


def vbatched_tuning(dtype: torch.dtype = torch.float64) -> dict:
    """The panel width and update tile the variable-size kernel uses per size bin."""
    nb, tile = (C.c_int * 8)(), (C.c_int * 8)()
    _check(getattr(_L.load(), f"magma_{_tune_prefix(dtype)}vbatched_tuning_get")(nb, tile),
           "vbatched_tuning_get")
    return _tune_dict(nb, tile)


def set_vbatched_tuning(nb, tile, dtype: torch.dtype = torch.float64) -> None:
    """Replace the table: nb and tile are 8-entry sequences (tile as index or name)."""
    t = [TILES.index(x) if isinstance(x, str) else int(x) for x in tile]
    nba, tia = (C.c_int * 8)(*[int(x) for x in nb]), (C.c_int * 8)(*t)
    _check(getattr(_L.load(), f"magma_{_tune_prefix(dtype)}vbatched_tuning_set")(nba, tia),
           "vbatched_tuning_set")


def autotune_vbatched(max_n: int, dtype: torch.dtype = torch.float64,
                      queue: Queue | None = None) -> dict:
    """Time every candidate per size bin up to max_n on the current device and install the
    fastest (magma_?getrf_vbatched_autotune).  Returns the table."""
    q = queue or Queue.current()
    nb, tile = (C.c_int * 8)(), (C.c_int * 8)()
    rc = getattr(_L.load(), f"magma_{_tune_prefix(dtype)}getrf_vbatched_autotune")(
        int(max_n), nb, tile, q.handle)
    _check(rc, "getrf_vbatched_autotune")
    return _tune_dict(nb, tile)


# fixed-size factorisation tuning (magma_?getrf_batched_autotune / _tuning_get / _set) and
# the tuning file (magma_lu_tuning_save / _load)
FIXED_TUNE_BINS = ("<=64", "<=128", "<=256", "<=512", "<=1024", ">1024")


def getrf_batched_tuning(dtype: torch.dtype = torch.float32) -> dict:
    """The fixed-size table of one precision: {bin: {two_level, band_ctas, tile64}}."""
    a, b, c = (C.c_int * 6)(), (C.c_int * 6)(), (C.c_int * 6)()
    rc = getattr(_L.load(), f"magma_{_tune_prefix(dtype)}getrf_batched_tuning_get")(a, b, c)
    _check(rc, "getrf_batched_tuning_get")
    return {k: {"two_level": a[i], "band_ctas": b[i], "tile64": c[i]}
            for i, k in enumerate(FIXED_TUNE_BINS)}


def set_getrf_batched_tuning(two_level, band_ctas, tile64, dtype: torch.dtype = torch.float32) -> None:
    arr = lambda v: (C.c_int * 6)(*[int(x) for x in v])
    rc = getattr(_L.load(), f"magma_{_tune_prefix(dtype)}getrf_batched_tuning_set")(
        arr(two_level), arr(band_ctas), arr(tile64))
    _check(rc, "getrf_batched_tuning_set")


def autotune_getrf_batched(max_n: int, batch: int, dtype: torch.dtype = torch.float32,
                           queue: Queue | None = None) -> dict:
    """Time the fixed-size candidates of every bin up to max_n on `batch` trial matrices and
    install the fastest (magma_?getrf_batched_autotune).  Returns the table."""
    q = queue or Queue.current()
    rc = getattr(_L.load(), f"magma_{_tune_prefix(dtype)}getrf_batched_autotune")(
        int(max_n), int(batch), q.handle)
    _check(rc, "getrf_batched_autotune")
    return getrf_batched_tuning(dtype)


def save_tuning(path) -> None:
    """Write both precisions' fixed-size and variable-size tables as JSON."""
    _check(_L.load().magma_lu_tuning_save(str(path).encode()), "magma_lu_tuning_save")


def load_tuning(path) -> None:
    """Install the tables of a file written by save_tuning (checked as a whole first)."""
    _check(_L.load().magma_lu_tuning_load(str(path).encode()), "magma_lu_tuning_load")
