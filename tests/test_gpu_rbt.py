"""Random butterfly transformation (magma_dgerbt_batched, magmablas_dprbt_*_batched)
and the RBT solve (magma_dgesv_rbt_batched): the transforms bit-identical to the
oracle's restatement for even and odd orders, generated butterflies in the
reference's range, and solutions accurate for matrices that need pivoting (a
zero leading entry) where LU without pivoting alone fails."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, ptr_array
from tests.util import scaled_residual

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _dbl(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 33, 100, 257])
def test_gerbt_matches_oracle(cuda, n):
    batch, nrhs, ld = 3, 2, n + 2
    rng = np.random.default_rng(n)
    S = rng.uniform(-1, 1, (batch, n, ld))
    B = rng.uniform(-1, 1, (batch, nrhs, ld))
    U = np.exp((rng.uniform(0, 1, 2 * n) - 0.5) / 10)
    V = np.exp((rng.uniform(0, 1, 2 * n) - 0.5) / 10)
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(B.copy()).to(cuda)
    lib = L.load()
    q = Queue.current(cuda).handle
    info = C.c_int(0)
    pS, pB = ptr_array(dS), ptr_array(dB)          # pointer arrays alive during the calls
    rc = lib.magma_dgerbt_batched(0, n, nrhs, _vp(pS), ld, _vp(pB), ld, U.ctypes.data,
                                  V.ctypes.data, C.byref(info), batch, q)
    assert rc == 0 and info.value == 0
    gS, gB = dS.cpu().numpy(), dB.cpu().numpy()
    for k in range(batch):
        rS, rB = S[k].copy(), B[k].copy()
        oracle.rbt_matrix(rS, U, V)
        oracle.rbt_vectors(True, rB, U, n)
        assert np.array_equal(gS[k], rS), k
        assert np.array_equal(gB[k], rB), k
    # x = V y on the device
    dv = torch.from_numpy(V).to(cuda)
    dY = torch.from_numpy(B.copy()).to(cuda)
    pY = ptr_array(dY)
    lib.magmablas_dprbt_mv_batched(n, nrhs, _vp(dv), _vp(pY), ld, batch, q)
    torch.cuda.synchronize()
    gY = dY.cpu().numpy()
    for k in range(batch):
        rY = B[k].copy()
        oracle.rbt_vectors(False, rY, V, n)
        assert np.array_equal(gY[k], rY), k


def test_gerbt_generates_butterflies(cuda):
    n, ld = 16, 16
    dS = torch.zeros((1, n, ld), dtype=torch.float64, device=cuda)
    dB = torch.zeros((1, 1, ld), dtype=torch.float64, device=cuda)
    U, V = np.zeros(2 * n), np.zeros(2 * n)
    info = C.c_int(0)
    q = Queue.current(cuda).handle
    pS, pB = ptr_array(dS), ptr_array(dB)
    assert L.load().magma_dgerbt_batched(1, n, 1, _vp(pS), ld, _vp(pB), ld, U.ctypes.data,
                                         V.ctypes.data, C.byref(info), 1, q) == 0
    lo, hi = np.exp(-0.05), np.exp(0.05)
    assert np.all((U >= lo) & (U <= hi)) and np.all((V >= lo) & (V <= hi))
    assert len(set(U.tolist())) == 2 * n


@pytest.mark.parametrize("n", [2, 7, 64, 129, 300])
def test_gesv_rbt_solves_pivoting_cases(cuda, n):
    batch, nrhs, ld = 4, 3, n
    rng = np.random.default_rng(100 + n)
    M = rng.uniform(-1, 1, (batch, n, n)) + 2 * np.eye(n)
    M[:, 0, 0] = 0.0                 # LU without pivoting would divide by zero at step 1
    Bm = rng.uniform(-1, 1, (batch, n, nrhs))
    dS = torch.from_numpy(np.ascontiguousarray(M.transpose(0, 2, 1))).to(cuda)
    dB = torch.from_numpy(np.ascontiguousarray(Bm.transpose(0, 2, 1))).to(cuda)
    info = torch.full((batch,), -5, dtype=torch.int32, device=cuda)
    pS, pB = ptr_array(dS), ptr_array(dB)
    rc = L.load().magma_dgesv_rbt_batched(n, nrhs, _vp(pS), ld, _vp(pB), ld, _vp(info), batch,
                                          Queue.current(cuda).handle)
    assert rc == 0
    X = dB.cpu().numpy().transpose(0, 2, 1)
    assert (info.cpu().numpy() == 0).all()
    res = scaled_residual(M, X, Bm)
    # no pivoting: the RBT bounds element growth only in probability, so the bound is
    # looser than the pivoted tester's 30 (the same solve without the RBT gives NaN)
    assert np.isfinite(X).all()
    assert res.max() < 30 * n, res.max()


def test_rbt_argument_errors(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    info = C.c_int(0)
    assert lib.magma_dgesv_rbt_batched(-1, 1, None, 1, None, 1, None, 1, q) == -1
    assert lib.magma_dgesv_rbt_batched(4, 1, None, 3, None, 4, None, 1, q) == -4
    assert lib.magma_dgerbt_batched(2, 4, 1, None, 4, None, 4, None, None, C.byref(info), 1, q) == -1
    assert lib.magma_dgerbt_batched(0, 4, 1, None, 4, None, 3, None, None, C.byref(info), 1, q) == -7
