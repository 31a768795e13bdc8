"""GMRES-based refinement (magma_dxgesv_gmres_batched_work, solver
Magma_REFINE_IRGMSTRS = 922): each refinement iteration's correction is solved
by FP32 GMRES preconditioned with the low-precision factors.

Against the oracle's restatement (oracle_dsgesv_gmres) with FP32 factors the
factors, pivots and info are bit-identical (the same FP32 LU); the GMRES dot
products are summed in a different order (per thread then across the block on
the GPU, in index order in the oracle), so the solutions agree to FP64
accuracy (both scaled residuals <= 30, difference <= 1e-9 relative) and the
inner iteration counts to within a few.  With FP16/BF16 tensor-core factors,
where plain refinement falls back to FP64 once kappa * u > 1, GMRES
refinement converges without the fallback."""
import ctypes as C

import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from magma_gb300 import lib as L
from magma_gb300.batched import Queue
from magma_gb300.testing import svd_batch_torch
from tests.util import from_storage, scaled_residual, to_storage

pytestmark = pytest.mark.gpu


def _svd(batch, n, kappas, seed):
    return svd_batch_torch(batch, n, kappas, seed, device="cpu").numpy()


def _gpu(A, Bm, cuda, solver, precision="fp32", itermax=30, tol=0.0):
    S, Bs = to_storage(A), to_storage(Bm)
    dS, dB = torch.from_numpy(S).to(cuda), torch.from_numpy(Bs).to(cuda)
    X, ipiv, info, iters = mg.dsgesv_batched(dS, dB, itermax=itermax, tol=tol,
                                             precision=precision, solver=solver)
    torch.cuda.synchronize()
    return (from_storage(X.cpu().numpy(), A.shape[1]), ipiv.cpu().numpy(), info.cpu().numpy(),
            iters.cpu().numpy())


@pytest.mark.parametrize("tol", [0.0, 30.0])
@pytest.mark.parametrize("n,nrhs", [(20, 1), (64, 3), (130, 6), (512, 4)])
def test_gmres_matches_oracle(cuda, n, nrhs, tol):
    batch = 6 if n < 512 else 3
    kappas = ([1e2, 1e4, 1e6] * 2)[:batch]
    A = _svd(batch, n, kappas, seed=n + nrhs)
    Bm = np.random.default_rng(n).uniform(-1, 1, (batch, n, nrhs))
    X, ipiv, info, iters = _gpu(A, Bm, cuda, "gmres", tol=tol)
    rX, ripiv, rinfo, riters = oracle.dsgesv_gmres_batched(to_storage(A), to_storage(Bm), tol=tol)
    rX = from_storage(rX, n)
    assert np.array_equal(info, rinfo)
    assert np.array_equal(ipiv[:, :n], ripiv[:, :n])
    assert np.all(iters >= 0) and np.all(riters >= 0), (iters, riters)
    assert np.all(np.abs(iters - riters) <= 2 + riters // 4), (iters, riters)
    assert scaled_residual(A, X, Bm).max() <= 30
    assert scaled_residual(A, rX, Bm).max() <= 30
    # both stop inside the stopping rule's backward error, so they may differ by
    # up to about kappa times it (scaled residual <= 30: 30 n eps; the default
    # rule: sqrt(n) eps)
    eps = np.finfo(np.float64).eps
    bound = np.array(kappas) * (30.0 * n if tol > 0 else np.sqrt(n)) * eps * 4
    rel = np.abs(X - rX).max(axis=(1, 2)) / np.abs(rX).max(axis=(1, 2))
    assert np.all(rel <= bound), (rel, bound)


@pytest.mark.parametrize("precision,kappa,ir_fails", [("fp16", 1e4, False), ("bf16", 1e4, True)])
def test_gmres_converges_from_tensor_core_factors(cuda, precision, kappa, ir_fails):
    """kappa * u near or above 1: GMRES refinement converges without the FP64
    fallback; with BF16 factors at kappa 1e4 plain refinement needs it.  (At
    kappa 1e6 neither converges from FP16 or BF16 factors on GB300 and the
    fallback solves in FP64: the FP32 inner solver's A32 and a GMRES(50) that
    barely reduces the preconditioned residual leave too little contraction.)"""
    n, batch, nrhs = 256, 4, 2
    A = _svd(batch, n, [kappa] * batch, seed=int(np.log10(kappa)) + (7 if precision == "bf16" else 0))
    Bm = np.random.default_rng(3).uniform(-1, 1, (batch, n, nrhs))
    Xg, _, infog, itg = _gpu(A, Bm, cuda, "gmres", precision)
    Xi, _, infoi, iti = _gpu(A, Bm, cuda, "ir", precision)
    assert np.all(infog == 0) and np.all(infoi == 0)
    assert np.all(itg >= 0), itg                     # converged without the fallback
    if ir_fails:
        assert np.any(iti < 0), iti                  # plain refinement fell back
    assert scaled_residual(A, Xg, Bm).max() <= 30
    assert scaled_residual(A, Xi, Bm).max() <= 30    # the fallback's FP64 solution


def test_solver_920_is_the_plain_refinement(cuda):
    A = _svd(3, 100, [1e2, 1e4, 1e6], seed=4)
    Bm = np.random.default_rng(4).uniform(-1, 1, (3, 100, 2))
    a = _gpu(A, Bm, cuda, "ir")
    S = to_storage(A)
    rX, ripiv, rinfo, riters = oracle.dsgesv_batched(S, to_storage(Bm))
    assert np.array_equal(a[0], from_storage(rX, 100))
    assert np.array_equal(a[3], riters)


def test_gmres_argument_errors(cuda):
    lib = L.load()
    q = Queue.current(cuda).handle
    lw = C.c_size_t(0)

    def call(prec, solver, n, nrhs):
        return lib.magma_dxgesv_gmres_batched_work(prec, solver, n, nrhs, None, max(n, 1), None,
                                                   None, max(n, 1), None, max(n, 1), None, None,
                                                   30, 0.0, 0, None, C.byref(lw), 1, q)

    assert call(901, 922, 4, 1) == -1
    assert call(900, 921, 4, 1) == -2
    assert call(900, 922, 4, 9) == -4
    assert call(900, 922, -1, 1) == -3
    assert call(900, 922, 4, 8) == 0 and lw.value > 0
    assert call(900, 920, 4, 16) == 0
