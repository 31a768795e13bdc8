"""Mixed-precision SPD refinement (magma_dsposv_batched_work): FP32 Cholesky,
FP64 residual, update and stopping rule, FP64 posv fallback.  Solutions,
iteration codes and info are bit-identical to the oracle's restatement
(oracle_dsposv); an SPD matrix whose FP32 Cholesky fails (iter -3) is solved
by the FP64 fallback; MagmaUpper and bad arguments are rejected."""
import ctypes as C

import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue
from tests.util import from_storage, scaled_residual, to_storage

pytestmark = pytest.mark.gpu


def _spd(batch, n, kappas, seed):
    """Q diag(s) Q^T with s geometric from 1 down to 1/kappa."""
    rng = np.random.default_rng(seed)
    out = np.empty((batch, n, n))
    for k in range(batch):
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        s = np.geomspace(1.0, 1.0 / kappas[k], n)
        M = (Q * s) @ Q.T
        out[k] = (M + M.T) / 2
    return out


@pytest.mark.parametrize("tol", [0.0, 30.0])
@pytest.mark.parametrize("n,nrhs", [(20, 1), (64, 3), (150, 6), (300, 4)])
def test_dsposv_matches_oracle(cuda, n, nrhs, tol):
    kappas = [1e2, 1e4, 1e6, 1e2, 1e4, 1e6]
    A = _spd(6, n, kappas, seed=n + nrhs)
    Bm = np.random.default_rng(n).uniform(-1, 1, (6, n, nrhs))
    S, Bs = to_storage(A), to_storage(Bm)
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(Bs).to(cuda)
    X, info, iters = mg.dsposv_batched(dS, dB, tol=tol)
    torch.cuda.synchronize()
    rX, rinfo, riters = oracle.dsposv_batched(S.copy(), Bs, tol=tol)
    assert np.array_equal(iters.cpu().numpy(), riters), (iters, riters)
    assert np.array_equal(info.cpu().numpy(), rinfo)
    assert np.array_equal(X.cpu().numpy(), rX)
    assert np.all(riters >= 0)
    assert scaled_residual(A, from_storage(rX, n), Bm).max() <= 30


def test_dsposv_fp32_cholesky_failure_falls_back(cuda):
    """kappa 1e12: FP32 Cholesky meets a non-positive pivot (iter -3), FP64 posv solves."""
    n = 96
    A = _spd(3, n, [1e12, 1e2, 1e12], seed=5)
    Bm = np.random.default_rng(5).uniform(-1, 1, (3, n, 2))
    S, Bs = to_storage(A), to_storage(Bm)
    dS, dB = torch.from_numpy(S.copy()).to(cuda), torch.from_numpy(Bs).to(cuda)
    X, info, iters = mg.dsposv_batched(dS, dB)
    torch.cuda.synchronize()
    rS = S.copy()
    rX, rinfo, riters = oracle.dsposv_batched(rS, Bs)
    it = iters.cpu().numpy()
    assert np.array_equal(it, riters)
    assert np.array_equal(X.cpu().numpy(), rX)
    assert np.array_equal(dS.cpu().numpy(), rS)       # fallback matrices hold their FP64 factor
    assert it[1] >= 0 and it[0] < 0 and it[2] < 0
    assert np.all(info.cpu().numpy() == 0)


def test_dsposv_argument_errors(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    lw = C.c_size_t(0)

    def call(uplo, n, nrhs, ld):
        return lib.magma_dsposv_batched_work(uplo, n, nrhs, None, ld, None, ld, None, ld, None,
                                             None, 30, 0.0, 0, None, C.byref(lw), 1, q)

    assert call(121, 4, 1, 4) == -1
    assert call(122, -1, 1, 4) == -2
    assert call(122, 4, 17, 4) == -3
    assert call(122, 4, 1, 3) == -5
    assert call(122, 4, 1, 4) == 0 and lw.value > 0
