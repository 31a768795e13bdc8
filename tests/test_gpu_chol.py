"""Batched Cholesky (magma_?potrf_batched, magma_?potrs_batched,
magma_?posv_batched, lower): factors and solutions bit-identical to the
oracle's restatement for orders inside one 32-column panel, across panels and
odd, padded leading dimensions, more right-hand sides than one solve block; a
matrix that is not positive definite reports the failing column in info and is
left where the factorisation stopped; MagmaUpper and bad arguments rejected
with MAGMA's codes."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue, ptr_array
from tests.util import scaled_residual

pytestmark = pytest.mark.gpu

LOWER, UPPER = 122, 121


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _spd(rng, batch, n, ld, npdt):
    """SPD matrices G G^T + n I in column-major storage (batch, n, ld)."""
    G = rng.uniform(-1, 1, (batch, n, n))
    M = G @ np.transpose(G, (0, 2, 1)) + n * np.eye(n)
    S = np.zeros((batch, n, ld))
    S[:, :, :n] = np.transpose(M, (0, 2, 1))
    return S.astype(npdt), M


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n", [1, 5, 32, 33, 64, 100, 257])
def test_posv_matches_oracle(cuda, dtype, n):
    batch, ld, nrhs = 4, n + 1, 3
    rng = np.random.default_rng(n)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    S, M = _spd(rng, batch, n, ld, npdt)
    fail_col = min(40, n // 2)
    S[1, fail_col, fail_col] = -1.0                # not positive definite at fail_col
    S[2, 0, 0] = np.nan                            # NaN pivot: info 1
    B = rng.uniform(-1, 1, (batch, nrhs, ld)).astype(npdt)
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(B.copy()).to(cuda)
    info = torch.full((batch,), -9, dtype=torch.int32, device=cuda)
    p = "d" if dtype == torch.float64 else "s"
    lib = L.load()
    q = Queue.current(cuda).handle
    pS, pB = ptr_array(dS), ptr_array(dB)
    assert getattr(lib, f"magma_{p}posv_batched")(LOWER, n, nrhs, _vp(pS), ld, _vp(pB), ld,
                                                  _vp(info), batch, q) == 0
    torch.cuda.synchronize()
    gS, gB, ginfo = dS.cpu().numpy(), dB.cpu().numpy(), info.cpu().numpy()
    for k in range(batch):
        rS, rB = S[k].copy(), B[k].copy()
        rinfo = oracle.potrf(rS)
        oracle.potrs(rS, rB)
        assert ginfo[k] == rinfo, (k, ginfo[k], rinfo)
        assert np.array_equal(gS[k], rS, equal_nan=True), k
        assert np.array_equal(gB[k], rB, equal_nan=True), k
    assert ginfo[0] == 0 and ginfo[3] == 0
    assert ginfo[1] == fail_col + 1
    assert ginfo[2] == 1
    # the strictly upper triangle is never written
    for k in range(batch):
        iu = np.triu_indices(n, 1)
        assert np.array_equal(gS[k][iu[1], iu[0]], S[k][iu[1], iu[0]], equal_nan=True)
    if dtype == torch.float64:
        X = np.transpose(gB[[0, 3], :, :n], (0, 2, 1))
        Bm = np.transpose(B[[0, 3], :, :n], (0, 2, 1))
        assert scaled_residual(M[[0, 3]], X, Bm).max() < 30


@pytest.mark.parametrize("n", [7, 96, 600])
def test_potrf_potrs_separately(cuda, n):
    """potrf then potrs with five right-hand sides (two solve blocks), batch of 3."""
    batch, ld, nrhs = 3, n + 3, 5
    rng = np.random.default_rng(100 + n)
    S, M = _spd(rng, batch, n, ld, np.float64)
    B = rng.uniform(-1, 1, (batch, nrhs, ld))
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(B.copy()).to(cuda)
    info = torch.full((batch,), -9, dtype=torch.int32, device=cuda)
    lib = L.load()
    q = Queue.current(cuda).handle
    pS, pB = ptr_array(dS), ptr_array(dB)
    assert lib.magma_dpotrf_batched(LOWER, n, _vp(pS), ld, _vp(info), batch, q) == 0
    assert lib.magma_dpotrs_batched(LOWER, n, nrhs, _vp(pS), ld, _vp(pB), ld, batch, q) == 0
    torch.cuda.synchronize()
    gS, gB = dS.cpu().numpy(), dB.cpu().numpy()
    assert (info.cpu().numpy() == 0).all()
    for k in range(batch):
        rS, rB = S[k].copy(), B[k].copy()
        assert oracle.potrf(rS) == 0
        oracle.potrs(rS, rB)
        assert np.array_equal(gS[k], rS), k
        assert np.array_equal(gB[k], rB), k
    Lm = np.tril(np.transpose(gS[:, :, :n], (0, 2, 1)))
    err = np.abs(Lm @ np.transpose(Lm, (0, 2, 1)) - M).max() / np.abs(M).max()
    assert err < 1e-14 * n


def test_chol_errors_and_empty(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    assert lib.magma_dpotrf_batched(UPPER, 4, None, 4, None, 1, q) == -1
    assert lib.magma_dpotrf_batched(LOWER, -1, None, 4, None, 1, q) == -2
    assert lib.magma_dpotrf_batched(LOWER, 4, None, 3, None, 1, q) == -4
    assert lib.magma_dpotrf_batched(LOWER, 4, None, 4, None, -1, q) == -6
    assert lib.magma_dpotrs_batched(UPPER, 4, 1, None, 4, None, 4, 1, q) == -1
    assert lib.magma_dpotrs_batched(LOWER, 4, -1, None, 4, None, 4, 1, q) == -3
    assert lib.magma_dpotrs_batched(LOWER, 4, 1, None, 3, None, 4, 1, q) == -5
    assert lib.magma_dpotrs_batched(LOWER, 4, 1, None, 4, None, 3, 1, q) == -7
    assert lib.magma_sposv_batched(UPPER, 4, 1, None, 4, None, 4, None, 1, q) == -1
    assert lib.magma_sposv_batched(LOWER, 4, 1, None, 4, None, 3, None, 1, q) == -7
    # empty problems launch nothing
    assert lib.magma_dpotrf_batched(LOWER, 0, None, 1, None, 5, q) == 0
    assert lib.magma_dposv_batched(LOWER, 4, 0, None, 4, None, 4, None, 5, q) == 0
    assert lib.magma_dposv_batched(LOWER, 4, 1, None, 4, None, 4, None, 0, q) == 0
