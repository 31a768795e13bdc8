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


def _buffers(S, B, cuda):
    b, n, ld = S.shape
    X = torch.empty_like(B)
    ipiv = torch.empty((b, n), dtype=torch.int32, device=cuda)
    info = torch.empty((b,), dtype=torch.int32, device=cuda)
    iters = torch.empty((b,), dtype=torch.int32, device=cuda)
    return {"S": S, "B": B, "X": X, "ipiv": ipiv, "info": info, "iters": iters,
            "dA": ptr_array(S), "dP": ptr_array(ipiv), "dB": ptr_array(B), "dX": ptr_array(X)}


def _call(buf, queue):
    b, n, ld = buf["S"].shape
    nrhs, ldb = buf["B"].shape[1], buf["B"].shape[2]
    rc = L.load().magma_dsgesv_batched_noalloc(n, nrhs, _vp(buf["dA"]), ld, _vp(buf["dP"]),
                                               _vp(buf["dB"]), ldb, _vp(buf["dX"]), buf["X"].shape[2],
                                               _vp(buf["info"]), _vp(buf["iters"]), b, queue.handle)
    torch.cuda.synchronize()
    return rc


def _noalloc(S, B, cuda):
    buf = _buffers(S, B, cuda)
    rc = _call(buf, Queue.current(cuda))
    return rc, buf["X"], buf["ipiv"], buf["info"], buf["iters"]


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


def test_noalloc_leaves_free_device_memory_unchanged(cuda):
    """The defining property: a successful call allocates nothing, neither in the call
    nor in the queue (a fresh queue, whose workspace stays empty)."""
    S, B = _inputs(13, 32, 80, 2, cuda)
    buf = _buffers(S.clone(), B, cuda)
    q = Queue(cuda.index or 0, torch.cuda.current_stream(cuda).cuda_stream)
    assert _call(buf, q) == 0             # first call on the device: symbol lookup, module loads
    buf["S"].copy_(S)
    free0 = torch.cuda.mem_get_info(cuda)[0]
    assert _call(buf, q) == 0
    free1 = torch.cuda.mem_get_info(cuda)[0]
    assert free1 == free0
    assert int(buf["iters"].min()) >= 0


def test_noalloc_rejects_batches_beyond_the_scratch(cuda, capfd):
    # 512 matrices of n = 512 need about 0.5 GiB of scratch, far above the fixed array;
    # the size is refused on the host before any pointer is read, so every entry of the
    # pointer arrays names the same small matrix
    need = mg.dsgesv_workspace_bytes(512, 4, 512)
    assert need > (32 << 20)
    A1 = torch.zeros((1, 512, 512), dtype=torch.float64, device=cuda)
    B1 = torch.zeros((1, 4, 512), dtype=torch.float64, device=cuda)
    buf = _buffers(A1.expand(512, 512, 512), B1.expand(512, 4, 512), cuda)   # stride 0: aliases
    assert int(buf["dA"].min()) == int(buf["dA"].max()) == A1.data_ptr()
    rc = _call(buf, Queue.current(cuda))
    assert rc == -103
    assert "static scratch" in capfd.readouterr().err
