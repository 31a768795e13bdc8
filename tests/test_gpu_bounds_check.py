"""The bounds-check build: the hot kernels' global accesses checked on the GPU.

libmagma_lu_bc.so is the library compiled with -DMLU_BOUNDS_CHECK: every
instrumented access (the rank-128 update's gathers, displaced rows, tile loads
and stores, the band kernel's pivot rows and strips, the deferred interchanges'
sources and destinations, the pivot indices of the small solve and of the
refinement's permutation) first checks that its row and column lie inside the
operand, records the first violation and skips the access.  The refinement
workload's routines run through it at the ragged sizes of the kernels' tiles
and panels; the record must stay empty and every result must equal the oracle
bit for bit.  The library is built on first use (about two minutes of nvcc).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import ptr_array

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bc(cuda):
    lib = L.load_bounds_checked()
    h = C.c_void_p()
    s = torch.cuda.current_stream(cuda)
    lib.magma_queue_create_from_cuda_internal(cuda.index or 0, C.c_void_p(s.cuda_stream), None, None,
                                              C.byref(h), b"bc", b"test", 0)
    assert h.value
    first, count = C.c_ulonglong(), C.c_ulonglong()
    assert lib.mlu_bounds_check_read(C.byref(first), C.byref(count), 1) == 0
    yield lib, h
    lib.magma_queue_destroy_internal(h, b"bc", b"test", 0)


def _record(lib):
    first, count = C.c_ulonglong(), C.c_ulonglong()
    assert lib.mlu_bounds_check_read(C.byref(first), C.byref(count), 1) == 0
    v = first.value
    return count.value, (v >> 48, (v >> 24) & 0xffffff, v & 0xffffff)


def _vp(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("m,n,batch", [(257, 257, 320), (300, 129, 320), (129, 300, 320), (512, 512, 160),
                                       (513, 400, 5), (1000, 999, 2), (65, 640, 4), (160, 161, 5)])
def test_sgetrf_within_bounds(cuda, bc, m, n, batch):
    lib, q = bc
    rng = np.random.default_rng(m * 3 + n)
    A = rng.uniform(-1, 1, (batch, n, m + 3)).astype(np.float32)
    S = torch.from_numpy(A).to(cuda)
    ipiv = torch.zeros((batch, min(m, n)), dtype=torch.int32, device=cuda)
    info = torch.zeros((batch,), dtype=torch.int32, device=cuda)
    dA, dP = ptr_array(S), ptr_array(ipiv)
    assert lib.magma_sgetrf_batched(m, n, _vp(dA), m + 3, _vp(dP), _vp(info), batch, q) == 0
    torch.cuda.synchronize()
    count, where = _record(lib)
    assert count == 0, f"{count} out-of-bounds accesses, first (site, row, col) = {where}"
    rA = A.copy()
    rp, ri = oracle.sgetrf_batched(rA, m)
    assert np.array_equal(S.cpu().numpy(), rA)
    assert np.array_equal(ipiv.cpu().numpy(), rp[:, :min(m, n)])
    assert np.array_equal(info.cpu().numpy(), ri)


@pytest.mark.parametrize("n", [1, 2, 7, 17, 31, 32, 33, 64, 65, 129])
def test_dgesv_within_bounds(cuda, bc, n):
    lib, q = bc
    batch, nrhs = 33, 2
    rng = np.random.default_rng(n)
    A = rng.uniform(-1, 1, (batch, n, n))
    B = rng.uniform(-1, 1, (batch, nrhs, n))
    S, X = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    ipiv = torch.zeros((batch, n), dtype=torch.int32, device=cuda)
    info = torch.zeros((batch,), dtype=torch.int32, device=cuda)
    dA, dP, dB = ptr_array(S), ptr_array(ipiv), ptr_array(X)
    assert lib.magma_dgesv_batched(n, nrhs, _vp(dA), n, _vp(dP), _vp(dB), n, _vp(info), batch, q) == 0
    torch.cuda.synchronize()
    count, where = _record(lib)
    assert count == 0, f"{count} out-of-bounds accesses, first (site, row, col) = {where}"
    rA, rB = A.copy(), B.copy()
    rp, ri = oracle.dgesv_batched(rA, rB)
    assert np.array_equal(S.cpu().numpy(), rA)
    assert np.array_equal(X.cpu().numpy(), rB)
    assert np.array_equal(ipiv.cpu().numpy(), rp)


@pytest.mark.parametrize("n,batch", [(300, 320), (512, 64), (129, 33)])
def test_refinement_within_bounds(cuda, bc, n, batch):
    lib, q = bc
    nrhs = 4
    rng = np.random.default_rng(n + batch)
    A = rng.uniform(-1, 1, (batch, n, n))
    A[1] = 0.0                                # a singular matrix: the FP64 fallback
    B = rng.uniform(-1, 1, (batch, nrhs, n))
    S, Bd = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    X = torch.zeros_like(Bd)
    ipiv = torch.zeros((batch, n), dtype=torch.int32, device=cuda)
    info = torch.zeros((batch,), dtype=torch.int32, device=cuda)
    it = torch.zeros((batch,), dtype=torch.int32, device=cuda)
    dA, dP, dB, dX = ptr_array(S), ptr_array(ipiv), ptr_array(Bd), ptr_array(X)
    assert lib.magma_dsgesv_batched(n, nrhs, _vp(dA), n, _vp(dP), _vp(dB), n, _vp(dX), n, _vp(info),
                                    _vp(it), batch, q) == 0
    torch.cuda.synchronize()
    count, where = _record(lib)
    assert count == 0, f"{count} out-of-bounds accesses, first (site, row, col) = {where}"
    rS = A.copy()
    rX, rp, rinfo, riters = oracle.dsgesv_batched(rS, B.copy())
    assert np.array_equal(it.cpu().numpy(), riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    assert np.array_equal(X.cpu().numpy(), rX, equal_nan=True)
    assert np.array_equal(S.cpu().numpy(), rS)
