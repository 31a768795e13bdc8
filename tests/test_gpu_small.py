"""GPU parity for n <= 32 (warp-per-matrix kernels) through the C ABI.

Bar: bit-identical to the CPU oracle (factors, pivots, info, solutions),
because both apply the same fused multiply-adds in the same order.  Covers
the reference tester's cases: ragged sizes, padded leading dimensions,
singular matrices (zeroed columns), exact pivot ties, NaN input, empty
batches, the transposed solve, and single precision.
"""
import numpy as np
import pytest
import torch

import magma_gb300 as mg
import oracle
from tests.util import scaled_residual, to_storage, from_storage

pytestmark = pytest.mark.gpu


def _run_gesv(S, X, cuda):
    dS = torch.from_numpy(S).to(cuda)
    dX = torch.from_numpy(X).to(cuda)
    ipiv, info = mg.gesv_batched(dS, dX)
    torch.cuda.synchronize()
    return dS.cpu().numpy(), dX.cpu().numpy(), ipiv.cpu().numpy(), info.cpu().numpy()


def _oracle_gesv(S, X):
    S, X = S.copy(), X.copy()
    f = oracle.dgesv_batched if S.dtype == np.float64 else oracle.sgesv_batched
    ipiv, info = f(S, X)
    return S, X, ipiv, info


def _assert_same(gpu, ref, n):
    S, X, ipiv, info = gpu
    rS, rX, ripiv, rinfo = ref
    assert np.array_equal(info, rinfo)
    assert np.array_equal(ipiv[:, :n], ripiv[:, :n])
    assert np.array_equal(S, rS, equal_nan=True)
    assert np.array_equal(X, rX, equal_nan=True)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("nrhs", [1, 2, 4, 5, 16])
@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 9, 16, 17, 24, 31, 32])
def test_gesv_small_bitexact(cuda, n, nrhs, dtype):
    rng = np.random.default_rng(1000 * n + nrhs)
    batch = 131
    S = to_storage(rng.uniform(-1, 1, (batch, n, n)).astype(dtype))
    X = to_storage(rng.uniform(-1, 1, (batch, n, nrhs)).astype(dtype))
    _assert_same(_run_gesv(S, X, cuda), _oracle_gesv(S, X), n)


def test_gesv_config1_shape_bitexact_and_accurate(cuda):
    """10,000 matrices 32x32, one RHS: the fused small path end to end."""
    rng = np.random.default_rng(1)
    A = rng.uniform(-1, 1, (10000, 32, 32))
    B = rng.uniform(-1, 1, (10000, 32, 1))
    S, X = to_storage(A), to_storage(B)
    gpu = _run_gesv(S, X, cuda)
    _assert_same(gpu, _oracle_gesv(S, X), 32)
    res = scaled_residual(A, from_storage(gpu[1], 32), B)
    assert res.max() < 30


def test_padded_leading_dimension(cuda):
    rng = np.random.default_rng(3)
    n, ld, nrhs = 20, 32, 3
    S = to_storage(rng.uniform(-1, 1, (50, n, n)), ld)
    X = to_storage(rng.uniform(-1, 1, (50, n, nrhs)), ld)
    S[:, :, n:] = 7.0                            # padding must be left untouched
    X[:, :, n:] = -3.0
    gpu = _run_gesv(S, X, cuda)
    ref = _oracle_gesv(S, X)
    _assert_same(gpu, ref, n)
    assert np.all(gpu[0][:, :, n:] == 7.0) and np.all(gpu[1][:, :, n:] == -3.0)


@pytest.mark.parametrize("n", [4, 16, 32])
def test_singular_info(cuda, n):
    rng = np.random.default_rng(5)
    A = rng.uniform(-1, 1, (9, n, n))
    A[:, :, 1] = 0.0
    A[:, :, n // 2] = 0.0
    A[0] = 0.0
    S, X = to_storage(A), to_storage(rng.uniform(-1, 1, (9, n, 2)))
    gpu = _run_gesv(S, X, cuda)
    ref = _oracle_gesv(S, X)
    assert np.array_equal(gpu[3], ref[3]) and np.all(gpu[3] > 0)
    assert np.array_equal(gpu[2], ref[2])
    assert np.array_equal(gpu[0], ref[0], equal_nan=True)


@pytest.mark.parametrize("n", [3, 6, 12, 32])
def test_exact_ties(cuda, n):
    rng = np.random.default_rng(9)
    A = rng.integers(-2, 3, (64, n, n)).astype(np.float64)
    B = rng.integers(-2, 3, (64, n, 1)).astype(np.float64)
    S, X = to_storage(A), to_storage(B)
    _assert_same(_run_gesv(S, X, cuda), _oracle_gesv(S, X), n)


def test_nan_input(cuda):
    rng = np.random.default_rng(2)
    A = rng.uniform(-1, 1, (8, 8, 8))
    A[0, 0, 0] = np.nan      # NaN on the diagonal: chosen as pivot
    A[1, 5, 0] = np.nan      # NaN below: never chosen
    A[2, 3, 4] = np.nan
    S, X = to_storage(A), to_storage(rng.uniform(-1, 1, (8, 8, 1)))
    _assert_same(_run_gesv(S, X, cuda), _oracle_gesv(S, X), 8)


@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("n", [1, 5, 16, 29, 32])
def test_getrf_getrs_small(cuda, n, trans):
    rng = np.random.default_rng(n)
    A = rng.uniform(-1, 1, (77, n, n))
    S = to_storage(A)
    B = to_storage(rng.uniform(-1, 1, (77, n, 6)))
    rS = S.copy()
    ripiv, rinfo = oracle.dgetrf_batched(rS)
    rB = B.copy()
    oracle.dgetrs_batched(rS, ripiv, rB, trans=trans)
    dS = torch.from_numpy(S).to(cuda)
    ipiv, info = mg.getrf_batched(dS)
    dB = torch.from_numpy(B).to(cuda)
    mg.getrs_batched(dS, ipiv, dB, trans=trans)
    torch.cuda.synchronize()
    assert np.array_equal(ipiv.cpu().numpy(), ripiv)
    assert np.array_equal(dS.cpu().numpy(), rS)
    assert np.array_equal(dB.cpu().numpy(), rB)


def test_empty_batch_and_zero_size(cuda):
    dS = torch.zeros((0, 4, 4), dtype=torch.float64, device=cuda)
    dX = torch.zeros((0, 1, 4), dtype=torch.float64, device=cuda)
    mg.gesv_batched(dS, dX)
    torch.cuda.synchronize()
