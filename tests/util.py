"""Shared helpers for the parity tests (numpy only)."""
from __future__ import annotations

import numpy as np

EPS = {np.float64: np.finfo(np.float64).eps, np.float32: np.finfo(np.float32).eps}


def to_storage(A: np.ndarray, ld: int | None = None) -> np.ndarray:
    """(batch, m, n) math orientation -> column-major storage (batch, n, ld)."""
    b, m, n = A.shape
    ld = m if ld is None else ld
    S = np.zeros((b, n, ld), dtype=A.dtype)
    S[:, :, :m] = np.transpose(A, (0, 2, 1))
    return S


def from_storage(S: np.ndarray, m: int) -> np.ndarray:
    return np.ascontiguousarray(np.transpose(S[:, :, :m], (0, 2, 1)))


def scaled_residual(A, X, B):
    """MAGMA tester metric ||B - A X||_inf / (||A||_inf ||X||_inf n eps) per matrix
    (testing/testing_zgesv_batched.cpp:131-152).  A (b,n,n), X and B (b,n,r)."""
    A = A.astype(np.float64)
    X = X.astype(np.float64)
    B = B.astype(np.float64)
    n = A.shape[1]
    eps = EPS[np.float64]
    R = A @ X - B
    # lange("I"): maximum absolute row sum
    rn = np.abs(R).sum(axis=2).max(axis=1)
    an = np.abs(A).sum(axis=2).max(axis=1)
    xn = np.abs(X).sum(axis=2).max(axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        return rn / (an * xn * n * eps)


def lu_error(A, LU, ipiv):
    """||P A - L U||_F / (||A||_F n), testing/testing_zgetrf_batched.cpp:41-80."""
    b, m, n = A.shape
    out = np.zeros(b)
    for k in range(b):
        PA = A[k].astype(np.float64).copy()
        for i, p in enumerate(ipiv[k][:min(m, n)]):
            p -= 1
            if p != i:
                PA[[i, p]] = PA[[p, i]]
        mn = min(m, n)
        L = np.tril(LU[k].astype(np.float64), -1)[:, :mn] + np.eye(m, mn)
        U = np.triu(LU[k].astype(np.float64))[:mn, :]
        out[k] = np.linalg.norm(PA - L @ U) / (np.linalg.norm(A[k]) * max(n, 1))
    return out


def explain_pivot_mismatch(A, ipiv_a, ipiv_b, rtol=1e-9):
    """For one matrix A (m, n), return (k, rel_gap) at the first step where the two
    pivot sequences differ, with rel_gap the relative difference of the two
    candidates' magnitudes in column k after k elimination steps (done with
    sequence ipiv_a).  A near-tie has rel_gap close to zero; a real
    disagreement has a large one.  Returns None when the sequences agree."""
    diff = np.nonzero(ipiv_a != ipiv_b)[0]
    if diff.size == 0:
        return None
    k = int(diff[0])
    W = A.astype(np.float64).copy()
    m, n = W.shape
    for t in range(k):
        p = ipiv_a[t] - 1
        W[[t, p]] = W[[p, t]]
        if W[t, t] != 0:
            W[t + 1:, t] /= W[t, t]
        W[t + 1:, t + 1:] -= np.outer(W[t + 1:, t], W[t, t + 1:])
    a = abs(W[ipiv_a[k] - 1, k])
    b = abs(W[ipiv_b[k] - 1, k])
    gap = abs(a - b) / max(a, b, np.finfo(np.float64).tiny)
    return k, gap
