"""LU without pivoting (magma_?getrf/getrs/gesv_nopiv_batched): bit-identical to
the oracle's restatement (the diagonal as pivot), including a zero diagonal
(info, column left unscaled), orders through the register and shared-memory
panels, padded leading dimensions, and both solve directions."""
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
@pytest.mark.parametrize("n", [5, 32, 33, 100, 600])
def test_nopiv_matches_oracle(cuda, dtype, n):
    batch, ld, nrhs = 4, n + 1, 3
    rng = np.random.default_rng(n)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    S = rng.uniform(-1, 1, (batch, n, ld)).astype(npdt)
    S[:, np.arange(n), np.arange(n)] += 4.0
    S[1, 0, 0] = 0.0                               # a zero pivot: info 1, column unscaled
    B = rng.uniform(-1, 1, (batch, nrhs, ld)).astype(npdt)
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(B.copy()).to(cuda)
    info = torch.full((batch,), -9, dtype=torch.int32, device=cuda)
    p = "d" if dtype == torch.float64 else "s"
    lib = L.load()
    q = Queue.current(cuda).handle
    dA, dX = ptr_array(dS), ptr_array(dB)
    assert getattr(lib, f"magma_{p}gesv_nopiv_batched")(n, nrhs, _vp(dA), ld, _vp(dX), ld,
                                                         _vp(info), batch, q) == 0
    torch.cuda.synchronize()
    gS, gB, ginfo = dS.cpu().numpy(), dB.cpu().numpy(), info.cpu().numpy()
    ident = np.arange(1, n + 1, dtype=np.int32)
    for k in range(batch):
        rS, rB = S[k].copy(), B[k].copy()
        rinfo = oracle.getrf_nopiv(rS)
        (oracle.dgetrs if p == "d" else oracle.sgetrs)(rS, ident, rB)
        assert ginfo[k] == rinfo, k
        assert np.array_equal(gS[k], rS, equal_nan=True), k
        assert np.array_equal(gB[k], rB, equal_nan=True), k
    assert ginfo[1] == 1
    # transposed solve with the factors
    dBt = torch.from_numpy(B.copy()).to(cuda)
    dXt = ptr_array(dBt)
    assert getattr(lib, f"magma_{p}getrs_nopiv_batched")(112, n, nrhs, _vp(dA), ld, _vp(dXt), ld,
                                                         None, batch, q) == 0
    torch.cuda.synchronize()
    gBt = dBt.cpu().numpy()
    for k in range(batch):
        rB = B[k].copy()
        (oracle.dgetrs if p == "d" else oracle.sgetrs)(gS[k].copy(), ident, rB, trans=True)
        assert np.array_equal(gBt[k], rB, equal_nan=True), k


def test_nopiv_rectangular_and_errors(cuda):
    rng = np.random.default_rng(3)
    lib = L.load()
    q = Queue.current(cuda).handle
    for m, n in [(70, 40), (40, 70)]:
        S = rng.uniform(-1, 1, (2, n, m)).astype(np.float64)
        for j in range(min(m, n)):
            S[:, j, j] += 4.0
        dS = torch.from_numpy(S.copy()).to(cuda)
        info = torch.empty((2,), dtype=torch.int32, device=cuda)
        dA = ptr_array(dS)
        assert lib.magma_dgetrf_nopiv_batched(m, n, _vp(dA), m, _vp(info), 2, q) == 0
        torch.cuda.synchronize()
        for k in range(2):
            r = S[k].copy()
            assert oracle.getrf_nopiv(r, m) == int(info[k])
            assert np.array_equal(dS[k].cpu().numpy(), r)
    assert lib.magma_dgetrf_nopiv_batched(-1, 4, None, 4, None, 1, q) == -1
    assert lib.magma_dgetrf_nopiv_batched(4, 4, None, 3, None, 1, q) == -4
    assert lib.magma_dgesv_nopiv_batched(4, 1, None, 4, None, 3, None, 1, q) == -6
    assert lib.magma_dgetrs_nopiv_batched(111, 4, 1, None, 3, None, 4, None, 1, q) == -5


def test_nopiv_band_path(cuda):
    """A batch large enough for the FP32 band kernel (no interchanges to resolve)."""
    n, batch, nrhs = 100, 320, 2
    rng = np.random.default_rng(31)
    S = rng.uniform(-1, 1, (batch, n, n)).astype(np.float32)
    S[:, np.arange(n), np.arange(n)] += 4.0
    B = rng.uniform(-1, 1, (batch, nrhs, n)).astype(np.float32)
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(B.copy()).to(cuda)
    info = torch.full((batch,), -9, dtype=torch.int32, device=cuda)
    lib = L.load()
    q = Queue.current(cuda).handle
    pS, pB = ptr_array(dS), ptr_array(dB)
    assert lib.magma_sgesv_nopiv_batched(n, nrhs, _vp(pS), n, _vp(pB), n, _vp(info), batch, q) == 0
    torch.cuda.synchronize()
    gS, gB = dS.cpu().numpy(), dB.cpu().numpy()
    assert (info.cpu().numpy() == 0).all()
    ident = np.arange(1, n + 1, dtype=np.int32)
    for k in range(0, batch, 37):
        rS, rB = S[k].copy(), B[k].copy()
        assert oracle.getrf_nopiv(rS) == 0
        oracle.sgetrs(rS, ident, rB)
        assert np.array_equal(gS[k], rS), k
        assert np.array_equal(gB[k], rB), k
