"""GPU parity for n > 32 (blocked panel / swap+TRSM / GEMM kernels, blocked
solves) through the C ABI, bit-identical to the CPU oracle.

Sizes straddle every blocking boundary (panel width 32, GEMM tile 64, solve
block 32), include rectangular getrf (m > n and m < n, like
testing/testing_zgetrf_batched.cpp), padded leading dimensions, singular
matrices, the transposed solve and single precision.
"""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from tests.util import from_storage, scaled_residual, to_storage

pytestmark = pytest.mark.gpu


def _gpu_getrf(S, m, cuda):
    dS = torch.from_numpy(S).to(cuda)
    ipiv, info = mg.getrf_batched(dS, m)
    torch.cuda.synchronize()
    return dS.cpu().numpy(), ipiv.cpu().numpy(), info.cpu().numpy()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [33, 40, 63, 64, 65, 96, 100, 128, 129, 200])
def test_getrf_square_bitexact(cuda, n, dtype):
    rng = np.random.default_rng(n)
    S = to_storage(rng.uniform(-1, 1, (5, n, n)).astype(dtype))
    rS = S.copy()
    f = oracle.dgetrf_batched if dtype == np.float64 else oracle.sgetrf_batched
    ripiv, rinfo = f(rS)
    gS, gipiv, ginfo = _gpu_getrf(S, n, cuda)
    assert np.array_equal(gipiv, ripiv)
    assert np.array_equal(ginfo, rinfo)
    assert np.array_equal(gS, rS)


@pytest.mark.parametrize("m,n", [(70, 33), (33, 70), (100, 64), (64, 100), (40, 8), (8, 40),
                                 (300, 45), (45, 300), (20, 24)])
def test_getrf_rectangular_bitexact(cuda, m, n):
    rng = np.random.default_rng(m * 1000 + n)
    S = to_storage(rng.uniform(-1, 1, (4, m, n)))
    rS = S.copy()
    ripiv, rinfo = oracle.dgetrf_batched(rS, m)
    gS, gipiv, ginfo = _gpu_getrf(S, m, cuda)
    assert np.array_equal(gipiv[:, :min(m, n)], ripiv[:, :min(m, n)])
    assert np.array_equal(gS, rS)


def test_getrf_padded_ld_and_singular(cuda):
    rng = np.random.default_rng(77)
    n, ld = 90, 128
    A = rng.uniform(-1, 1, (6, n, n))
    A[1, :, 3] = 0.0
    A[1, :, 50] = 0.0
    A[2] = 0.0
    A[3, :, 89] = 0.0
    S = to_storage(A, ld)
    S[:, :, n:] = 5.0
    rS = S.copy()
    ripiv, rinfo = oracle.dgetrf_batched(rS, n)
    gS, gipiv, ginfo = _gpu_getrf(S, n, cuda)
    assert np.array_equal(ginfo, rinfo)
    assert list(ginfo[:4]) == [0, 4, 1, 90]
    assert np.array_equal(gipiv, ripiv)
    assert np.array_equal(gS, rS)
    assert np.all(gS[:, :, n:] == 5.0)


@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("n,nrhs", [(33, 1), (64, 4), (100, 8), (129, 9), (256, 16), (75, 3)])
def test_getrs_bitexact(cuda, n, nrhs, trans):
    rng = np.random.default_rng(n + nrhs)
    S = to_storage(rng.uniform(-1, 1, (4, n, n)))
    B = to_storage(rng.uniform(-1, 1, (4, n, nrhs)))
    rS = S.copy()
    ripiv, _ = oracle.dgetrf_batched(rS)
    rB = B.copy()
    oracle.dgetrs_batched(rS, ripiv, rB, trans=trans)
    dS = torch.from_numpy(rS).to(cuda)
    dB = torch.from_numpy(B).to(cuda)
    mg.getrs_batched(dS, torch.from_numpy(ripiv).to(cuda), dB, trans=trans)
    torch.cuda.synchronize()
    assert np.array_equal(dB.cpu().numpy(), rB)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n,nrhs", [(64, 4), (512, 4), (257, 16)])
def test_gesv_bitexact_and_residual(cuda, n, nrhs, dtype):
    rng = np.random.default_rng(3 * n + nrhs)
    batch = 3
    A = rng.uniform(-1, 1, (batch, n, n)).astype(dtype)
    Bm = rng.uniform(-1, 1, (batch, n, nrhs)).astype(dtype)
    S, X = to_storage(A), to_storage(Bm)
    rS, rX = S.copy(), X.copy()
    f = oracle.dgesv_batched if dtype == np.float64 else oracle.sgesv_batched
    ripiv, rinfo = f(rS, rX)
    dS = torch.from_numpy(S).to(cuda)
    dX = torch.from_numpy(X).to(cuda)
    ipiv, info = mg.gesv_batched(dS, dX)
    torch.cuda.synchronize()
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(dS.cpu().numpy(), rS)
    assert np.array_equal(dX.cpu().numpy(), rX)
    if dtype == np.float64:
        res = scaled_residual(A, from_storage(dX.cpu().numpy(), n), Bm)
        assert res.max() < 30


def test_gesv_n1024_fp64(cuda):
    """Largest size of the serving workload: panel width shrinks to fit shared memory."""
    rng = np.random.default_rng(1024)
    n = 1024
    A = rng.uniform(-1, 1, (2, n, n))
    Bm = rng.uniform(-1, 1, (2, n, 2))
    S, X = to_storage(A), to_storage(Bm)
    rS, rX = S.copy(), X.copy()
    ripiv, _ = oracle.dgesv_batched(rS, rX)
    dS = torch.from_numpy(S).to(cuda)
    dX = torch.from_numpy(X).to(cuda)
    ipiv, info = mg.gesv_batched(dS, dX)
    torch.cuda.synchronize()
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(dX.cpu().numpy(), rX)
    assert np.array_equal(dS.cpu().numpy(), rS)


# Batches large enough for the fused band kernel (interchanges + TRSM + trailing
# update in one launch per step, at least two CTAs per SM): square, tall, wide
# (steps with no rows below the panel), padded ld with singular columns, FP32
# register panels of four rows per thread, m above the deferred-interchange
# limit, and steps that switch between the band kernel and the per-tile kernels
# as the bands run out.
@pytest.mark.parametrize("m,n,batch,dtype", [(100, 100, 320, np.float64),
                                             (100, 100, 320, np.float32),
                                             (300, 200, 160, np.float64),
                                             (150, 400, 160, np.float64),
                                             (520, 520, 48, np.float32),
                                             (1100, 64, 320, np.float64)])
def test_getrf_band_path_bitexact(cuda, m, n, batch, dtype):
    rng = np.random.default_rng(m + 7 * n + batch)
    S = to_storage(rng.uniform(-1, 1, (batch, m, n)).astype(dtype))
    rS = S.copy()
    f = oracle.dgetrf_batched if dtype == np.float64 else oracle.sgetrf_batched
    ripiv, rinfo = f(rS, m)
    gS, gipiv, ginfo = _gpu_getrf(S, m, cuda)
    k = min(m, n)
    assert np.array_equal(ginfo, rinfo)
    assert np.array_equal(gipiv[:, :k], ripiv[:, :k])
    assert np.array_equal(gS, rS)


def test_band_path_padded_ld_singular_and_solve(cuda):
    rng = np.random.default_rng(91)
    n, ld, batch = 90, 128, 320
    A = rng.uniform(-1, 1, (batch, n, n))
    A[1, :, 3] = 0.0
    A[2] = 0.0
    A[3, :, 89] = 0.0
    Bm = rng.uniform(-1, 1, (batch, n, 2))
    S, X = to_storage(A, ld), to_storage(Bm, ld)
    S[:, :, n:] = 5.0
    rS, rX = S.copy(), X.copy()
    ripiv, rinfo = oracle.dgesv_batched(rS, rX)
    dS, dX = torch.from_numpy(S).to(cuda), torch.from_numpy(X).to(cuda)
    ipiv, info = mg.gesv_batched(dS, dX)
    torch.cuda.synchronize()
    ginfo = info.cpu().numpy()
    assert np.array_equal(ginfo, rinfo)
    assert list(ginfo[:4]) == [0, 4, 1, 90]
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(dS.cpu().numpy(), rS)
    good = ginfo == 0
    assert np.array_equal(dX.cpu().numpy()[good], rX[good])
    assert np.all(dS.cpu().numpy()[:, :, n:] == 5.0)
