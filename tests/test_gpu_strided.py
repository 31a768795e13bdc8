"""Strided-batch entry points (magma_?getrf/getrs/gesv_batched_strided): one base
pointer and stride per operand; results identical to the pointer-array routines
(and so to the oracle), with strides larger than the matrices; argument errors."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n,nrhs", [(7, 2), (32, 1), (100, 5)])
def test_strided_gesv_and_getrf_match_oracle(cuda, dtype, n, nrhs):
    batch, ld, ldb = 6, n + 2, n + 1
    sA, sB, sP = ld * n + 17, ldb * nrhs + 5, n + 3          # strides beyond the data
    npdt = np.float64 if dtype == torch.float64 else np.float32
    rng = np.random.default_rng(n)
    A = rng.uniform(-1, 1, batch * sA).astype(npdt)
    B = rng.uniform(-1, 1, batch * sB).astype(npdt)
    dA, dB = torch.from_numpy(A.copy()).to(cuda), torch.from_numpy(B.copy()).to(cuda)
    dP = torch.zeros(batch * sP, dtype=torch.int32, device=cuda)
    info = torch.empty(batch, dtype=torch.int32, device=cuda)
    p = "d" if dtype == torch.float64 else "s"
    lib = L.load()
    q = Queue.current(cuda).handle
    rc = getattr(lib, f"magma_{p}gesv_batched_strided")(n, nrhs, _vp(dA), ld, sA, _vp(dP), sP,
                                                         _vp(dB), ldb, sB, _vp(info), batch, q)
    torch.cuda.synchronize()
    assert rc == 0
    gA, gB, gP = dA.cpu().numpy(), dB.cpu().numpy(), dP.cpu().numpy()
    for k in range(batch):
        S = A[k * sA:k * sA + ld * n].reshape(n, ld).copy()
        X = B[k * sB:k * sB + ldb * nrhs].reshape(nrhs, ldb).copy()
        ip, _ = (oracle.dgesv_batched if p == "d" else oracle.sgesv_batched)(S[None], X[None])
        assert np.array_equal(gA[k * sA:k * sA + ld * n].reshape(n, ld), S)
        assert np.array_equal(gB[k * sB:k * sB + ldb * nrhs].reshape(nrhs, ldb), X)
        assert np.array_equal(gP[k * sP:k * sP + n], ip[0][:n])
        # the gaps between matrices are untouched
        assert np.array_equal(gA[k * sA + ld * n:(k + 1) * sA], A[k * sA + ld * n:(k + 1) * sA])
    # getrs on the factors with the transposed system, against the oracle
    Bt = torch.from_numpy(B.copy()).to(cuda)
    rc = getattr(lib, f"magma_{p}getrs_batched_strided")(112, n, nrhs, _vp(dA), ld, sA, _vp(dP),
                                                         sP, _vp(Bt), ldb, sB, batch, q)
    torch.cuda.synchronize()
    assert rc == 0
    gBt = Bt.cpu().numpy()
    for k in range(batch):
        LU = gA[k * sA:k * sA + ld * n].reshape(n, ld).copy()
        X = B[k * sB:k * sB + ldb * nrhs].reshape(nrhs, ldb).copy()
        (oracle.dgetrs if p == "d" else oracle.sgetrs)(LU, gP[k * sP:k * sP + n].copy(), X,
                                                       trans=True)
        assert np.array_equal(gBt[k * sB:k * sB + ldb * nrhs].reshape(nrhs, ldb), X)
    # getrf alone on a fresh copy gives the same factors
    dA2 = torch.from_numpy(A.copy()).to(cuda)
    dP2 = torch.zeros_like(dP)
    rc = getattr(lib, f"magma_{p}getrf_batched_strided")(n, n, _vp(dA2), ld, sA, _vp(dP2), sP,
                                                         _vp(info), batch, q)
    torch.cuda.synchronize()
    assert rc == 0
    assert torch.equal(dA2, dA) and torch.equal(dP2, dP)


def test_strided_argument_errors(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    assert lib.magma_dgesv_batched_strided(8, 1, None, 8, 63, None, 8, None, 8, 8, None, 2, q) == -5
    assert lib.magma_dgesv_batched_strided(8, 1, None, 8, 64, None, 7, None, 8, 8, None, 2, q) == -7
    assert lib.magma_dgesv_batched_strided(8, 2, None, 8, 64, None, 8, None, 8, 15, None, 2, q) == -10
    assert lib.magma_dgetrf_batched_strided(8, 8, None, 8, 63, None, 8, None, 2, q) == -5
    assert lib.magma_dgetrs_batched_strided(111, 8, 1, None, 8, 64, None, 8, None, 8, 7, 2, q) == -11
