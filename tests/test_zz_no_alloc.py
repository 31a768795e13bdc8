"""magma_dsgesv_batched_noalloc: the refinement solve for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Checked through the C ABI against magma_dsgesv_batched_work with a
caller-provided workspace, on two calls in a row with different inputs: the
second call reuses the scratch the first one left behind.  The two entry
points run the same kernels, so the results must agree exactly (the bar of
every parity test here).  This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest
import torch

import magma_gb300 as mg
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, ptr_array
from magma_gb300.testing import svd_batch_torch

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _noalloc(S, B, cuda):
    b, n, ld = S.shape
    nrhs, ldb = B.shape[1], B.shape[2]
    X = torch.empty_like(B)
    ipiv = torch.empty((b, n), dtype=torch.int32, device=cuda)
    info = torch.empty((b,), dtype=torch.int32, device=cuda)
    iters = torch.empty((b,), dtype=torch.int32, device=cuda)
    dA, dP, dB, dX = ptr_array(S), ptr_array(ipiv), ptr_array(B), ptr_array(X)
    rc = L.load().magma_dsgesv_batched_noalloc(n, nrhs, _vp(dA), ld, _vp(dP), _vp(dB), ldb,
                                               _vp(dX), X.shape[2], _vp(info), _vp(iters), b,
                                               Queue.current(cuda).handle)
    torch.cuda.synchronize()
    return rc, X, ipiv, info, iters


def _inputs(seed, batch, n, nrhs, cuda):
    A = svd_batch_torch(batch, n, [1e2, 1e4, 1e6] * batch, seed, device="cpu")[:batch]
    Bm = torch.from_numpy(np.random.default_rng(seed).uniform(-1, 1, (batch, n, nrhs)))
    return (A.transpose(1, 2).contiguous().to(cuda), Bm.transpose(1, 2).contiguous().to(cuda))


def test_noalloc_matches_work_entry_two_calls(cuda):
    for call, (seed, batch, n, nrhs) in enumerate(((11, 24, 96, 4), (12, 40, 64, 3))):
        S, B = _inputs(seed, batch, n, nrhs, cuda)
        S_ref, B_ref = S.clone(), B.clone()
        rc, X, ipiv, info, iters = _noalloc(S, B, cuda)
        assert rc == 0, f"call {call}: magma_dsgesv_batched_noalloc returned {rc}"
        # existing entry point with its own workspace, same inputs
        Xr, ipivr, infor, itersr = mg.dsgesv_batched(S_ref, B_ref)
        torch.cuda.synchronize()
        assert torch.equal(iters, itersr), call
        assert torch.equal(info, infor), call
        assert torch.equal(ipiv, ipivr), call
        assert torch.equal(X, Xr), call
        assert torch.equal(S, S_ref) and torch.equal(B, B_ref)


def test_noalloc_rejects_batches_beyond_the_scratch(cuda, capfd):
    # 512 matrices of n = 512 need about 0.5 GiB of scratch, far above the fixed array
    need = mg.dsgesv_workspace_bytes(512, 4, 512)
    assert need > (32 << 20)
    S = torch.zeros((512, 512, 512), dtype=torch.float64, device=cuda)
    B = torch.zeros((512, 4, 512), dtype=torch.float64, device=cuda)
    rc = _noalloc(S, B, cuda)[0]
    assert rc == -103
    assert "static scratch" in capfd.readouterr().err
