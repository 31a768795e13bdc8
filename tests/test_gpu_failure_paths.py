"""Failure paths, exercised without faulting, trapping or hanging the GPU.

* Bounded device waits: the tensor-core kernels wait on mbarriers with a clock
  limit.  magma_sgetrf_batched_tc_wait_selftest runs the same wait on an
  mbarrier that nothing arrives at (nothing in flight), with a short limit; the
  wait must run out, record error 3, free its tensor memory and leave the
  context usable -- checked by a refinement solve right after it.
* Device allocation failure: magma_lu_fail_allocations makes the library's
  next allocations fail as if the device were out of memory; the routines that
  grow a queue workspace must return MAGMA_ERR_DEVICE_ALLOC (-113) as the
  reference does (src/zgetrf_batched.cpp:137-142), and succeed once the hook is
  off.
"""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, _vp, ptr_array
from magma_gb300.testing import svd_batch_torch

pytestmark = pytest.mark.gpu

MAGMA_ERR_DEVICE_ALLOC = -113


def _fresh_queue(cuda):
    return Queue(cuda.index or 0, torch.cuda.current_stream(cuda).cuda_stream)


def test_tensor_core_wait_runs_out_and_recovers(cuda):
    q = Queue.current(cuda)
    flag = torch.zeros(1, dtype=torch.int32, device=cuda)
    lib = L.load()
    for limit in (1000, 2_000_000):             # ~0.5 us and ~1 ms of SM clocks
        assert lib.magma_sgetrf_batched_tc_wait_selftest(limit, _vp(flag), q.handle) == 3
    assert int(flag.item()) == 3
    assert lib.magma_sgetrf_batched_tc_wait_selftest(0, _vp(flag), q.handle) == -1
    # the context still works: a small refinement solve, bit-exact with the oracle
    A = svd_batch_torch(4, 48, [1e2, 1e4, 1e6, 1e3], 5, device="cpu").numpy()
    B = np.random.default_rng(5).uniform(-1, 1, (4, 2, 48))
    S = np.ascontiguousarray(A.transpose(0, 2, 1))
    X, ipiv, info, iters = mg.dsgesv_batched(torch.from_numpy(S.copy()).to(cuda),
                                             torch.from_numpy(B).to(cuda))
    torch.cuda.synchronize()
    rX, _, _, riters = oracle.dsgesv_batched(S.copy(), B.copy())
    assert np.array_equal(iters.cpu().numpy(), riters)
    assert np.array_equal(X.cpu().numpy(), rX)


def test_tensor_core_factorisation_reports_no_timeout(cuda):
    """A real tensor-core factorisation leaves its error flag at 0."""
    b, n = 4, 256
    A = torch.rand((b, n, n), dtype=torch.float32, generator=torch.Generator().manual_seed(3)) - 0.5
    S = A.transpose(1, 2).contiguous().to(cuda)
    q = Queue.current(cuda)
    lib = L.load()
    import ctypes as C
    lw = C.c_size_t(0)
    assert lib.magma_sgetrf_batched_tc(930, n, n, None, n, None, None, None, C.byref(lw), b, q.handle) == 0
    work = torch.empty((lw.value,), dtype=torch.uint8, device=cuda)
    ipiv = torch.empty((b, n), dtype=torch.int32, device=cuda)
    info = torch.empty((b,), dtype=torch.int32, device=cuda)
    # the pointer arrays must outlive the call (a temporary's memory is reused at once)
    dA, dP = ptr_array(S), ptr_array(ipiv)
    rc = lib.magma_sgetrf_batched_tc(930, n, n, _vp(dA), n, _vp(dP), _vp(info), _vp(work), C.byref(lw),
                                     b, q.handle)
    assert rc == 0
    assert lib.magma_sgetrf_batched_tc_status(n, n, _vp(work), b, q.handle) == 0


def _dsgesv_args(cuda, b=3, n=40, nrhs=2):
    A = svd_batch_torch(b, n, [1e2] * b, 9, device="cpu")
    S = A.transpose(1, 2).contiguous().to(cuda)
    B = torch.from_numpy(np.random.default_rng(9).uniform(-1, 1, (b, nrhs, n))).to(cuda)
    X = torch.empty_like(B)
    ipiv = torch.empty((b, n), dtype=torch.int32, device=cuda)
    info = torch.empty((b,), dtype=torch.int32, device=cuda)
    iters = torch.empty((b,), dtype=torch.int32, device=cuda)
    keep = (S, B, X, ipiv, info, iters, ptr_array(S), ptr_array(ipiv), ptr_array(B), ptr_array(X))
    args = (n, nrhs, _vp(keep[6]), n, _vp(keep[7]), _vp(keep[8]), n, _vp(keep[9]), n, _vp(info),
            _vp(iters), b)
    return keep, args


def test_workspace_allocation_failure_returns_device_alloc(cuda):
    lib = L.load()
    keep, args = _dsgesv_args(cuda)
    q = _fresh_queue(cuda)                     # an empty queue workspace: the call must allocate
    try:
        assert lib.magma_lu_fail_allocations(1) == 0
        assert lib.magma_dsgesv_batched(*args, q.handle) == MAGMA_ERR_DEVICE_ALLOC
        assert lib.magma_lu_fail_allocations(0) == 0      # the one failure was used
    finally:
        lib.magma_lu_fail_allocations(0)
    assert lib.magma_dsgesv_batched(*args, q.handle) == 0
    torch.cuda.synchronize()
    assert int(keep[5].min()) >= 0             # converged


def test_vbatched_workspace_allocation_failure(cuda):
    lib = L.load()
    ns = [40, 70, 9]
    rng = np.random.default_rng(2)
    As = [rng.uniform(-1, 1, (n, n)) for n in ns]
    Bs = [rng.uniform(-1, 1, (1, n)) for n in ns]
    A = mg.VBatch([a.shape for a in As], ns, torch.float64, cuda).load(As)
    B = mg.VBatch([b.shape for b in Bs], ns, torch.float64, cuda).load(Bs)
    q = _fresh_queue(cuda)
    try:
        lib.magma_lu_fail_allocations(1)
        with pytest.raises(RuntimeError, match="-113"):
            mg.gesv_vbatched(A, B, queue=q)
    finally:
        lib.magma_lu_fail_allocations(0)
    A.load(As)
    B.load(Bs)
    mg.gesv_vbatched(A, B, queue=q)
    torch.cuda.synchronize()
    rA, rB = [a.copy() for a in As], [b.copy() for b in Bs]
    oracle.dgesv_vbatched(ns, [1] * 3, rA, rB)
    for k in range(3):
        assert np.array_equal(B.view(k).cpu().numpy(), rB[k])
