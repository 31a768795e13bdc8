"""Batched inverse from the LU factors (magma_?getri_outofplace_batched,
src/zgetri_outofplace_batched.cpp): bit-identical to the oracle's restatement,
within rounding of numpy's inverse, for orders around the 32-row block edges,
with padded leading dimensions; argument errors as MAGMA returns them."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, ptr_array

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 100, 257])
def test_getri_matches_oracle(cuda, dtype, n):
    batch, ld = 5, n + 3
    rng = np.random.default_rng(n)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    M = (4 * np.eye(n) + rng.uniform(-1, 1, (batch, n, n))).astype(npdt)   # math orientation
    S = np.zeros((batch, n, ld), dtype=npdt)
    S[:, :, :n] = M.transpose(0, 2, 1)
    dS = torch.from_numpy(S).to(cuda)
    ipiv = torch.empty((batch, n), dtype=torch.int32, device=cuda)
    info = torch.empty((batch,), dtype=torch.int32, device=cuda)
    lib = L.load()
    p = "d" if dtype == torch.float64 else "s"
    q = Queue.current(cuda).handle
    dA, dP = ptr_array(dS), ptr_array(ipiv)
    assert getattr(lib, f"magma_{p}getrf_batched")(n, n, _vp(dA), ld, _vp(dP), _vp(info), batch,
                                                   q) == 0
    Inv = torch.full((batch, n, n + 1), 7.0, dtype=dtype, device=cuda)
    dI = ptr_array(Inv)
    assert getattr(lib, f"magma_{p}getri_outofplace_batched")(n, _vp(dA), ld, _vp(dP), _vp(dI),
                                                              n + 1, _vp(info), batch, q) == 0
    torch.cuda.synchronize()
    LU, P, G = dS.cpu().numpy(), ipiv.cpu().numpy(), Inv.cpu().numpy()
    for k in range(batch):
        ref = oracle.getri(LU[k].copy(), P[k])
        assert np.array_equal(G[k][:, :n], ref), k
        assert np.all(G[k][:, n] == 7.0)                       # padding untouched
        inv = np.linalg.inv(M[k].astype(np.float64))
        tol = 64 * np.linalg.cond(M[k].astype(np.float64)) * np.finfo(npdt).eps
        assert np.abs(G[k][:, :n].T - inv).max() <= tol * np.abs(inv).max(), k


def test_getri_argument_errors(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    assert lib.magma_dgetri_outofplace_batched(-1, None, 1, None, None, 1, None, 1, q) == -1
    assert lib.magma_dgetri_outofplace_batched(4, None, 3, None, None, 4, None, 1, q) == -3
    assert lib.magma_dgetri_outofplace_batched(4, None, 4, None, None, 3, None, 1, q) == -6
    assert lib.magma_dgetri_outofplace_batched(0, None, 1, None, None, 1, None, 1, q) == 0
