"""Pin the oracle's restatements of the widened routines against independent
formulations: LU without pivoting (L U = A, zero-pivot info), the depth-2
random butterfly transformation (explicit butterfly matrices: U^T A V, U^T b,
V y, and the RBT solve identity), and Cholesky (LAPACK dpotrf/dpotrs through
scipy: same info for matrices that are not positive definite, factors and
solutions equal to rounding)."""
import numpy as np
import pytest

import oracle

RBT_C = 1.0 / np.sqrt(2.0)


def _level_blocks(level, n):
    """(start, order) of the butterflies of one level: one of order n at level 0,
    ceil(n/2) and the rest at level 1 (magma_dgerbt_batched's depth-2 RBT)."""
    if level == 0:
        return [(0, n)]
    n1 = (n + 1) // 2
    return [(0, n1), (n1, n - n1)]


def _butterfly(level, n, w):
    """The level's butterfly matrix B with (B x)_i = c (R x_i + S x_{i+g}),
    (B x)_{i+g} = c (R x_i - S x_{i+g}); an odd block's last index is fixed."""
    B = np.zeros((n, n))
    for b0, m in _level_blocks(level, n):
        g = m // 2
        base = 0 if level == 0 else n + b0
        for k in range(g):
            i, j = b0 + k, b0 + k + g
            R, S = w[base + k], w[base + k + g]
            B[i, i], B[i, j] = RBT_C * R, RBT_C * S
            B[j, i], B[j, j] = RBT_C * R, -RBT_C * S
        if m % 2:
            B[b0 + m - 1, b0 + m - 1] = 1.0
    return B


def _full(level_w, n):
    return _butterfly(1, n, level_w) @ _butterfly(0, n, level_w)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 33, 100])
def test_rbt_matches_explicit_butterflies(n):
    rng = np.random.default_rng(n)
    u = np.exp((rng.uniform(0, 1, 2 * n) - 0.5) / 10)
    v = np.exp((rng.uniform(0, 1, 2 * n) - 0.5) / 10)
    U, V = _full(u, n), _full(v, n)
    A = rng.uniform(-1, 1, (n, n))
    S = np.ascontiguousarray(A.T)
    oracle.rbt_matrix(S, u, v)
    np.testing.assert_allclose(S.T, U.T @ A @ V, rtol=0, atol=1e-13 * max(1, n))
    b = rng.uniform(-1, 1, (2, n))
    ub = oracle.rbt_vectors(True, b.copy(), u, n)
    np.testing.assert_allclose(ub, (U.T @ b.T).T, rtol=0, atol=1e-14 * max(1, n))
    vb = oracle.rbt_vectors(False, b.copy(), v, n)
    np.testing.assert_allclose(vb, (V @ b.T).T, rtol=0, atol=1e-14 * max(1, n))
    # the RBT solve: (U^T A V) y = U^T b, x = V y solves A x = b
    Ar = A + n * np.eye(n)
    Sr = np.ascontiguousarray(Ar.T)
    oracle.rbt_matrix(Sr, u, v)
    y = np.linalg.solve(Sr.T, oracle.rbt_vectors(True, b[:1].copy(), u, n)[0])
    x = oracle.rbt_vectors(False, y[None, :].copy(), v, n)[0]
    np.testing.assert_allclose(Ar @ x, b[0], rtol=0, atol=1e-12)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n", [(5, 5), (40, 40), (70, 40), (40, 70)])
def test_getrf_nopiv_reconstructs(dtype, m, n):
    rng = np.random.default_rng(m * 100 + n)
    A = rng.uniform(-1, 1, (m, n))
    for j in range(min(m, n)):
        A[j, j] += 4.0
    S = np.ascontiguousarray(A.T).astype(dtype)
    assert oracle.getrf_nopiv(S, m) == 0
    F = S.T.astype(np.float64)
    k = min(m, n)
    Lm = np.tril(F[:, :k], -1) + np.eye(m, k)
    Um = np.triu(F[:k, :])
    tol = 50 * np.finfo(dtype).eps * max(m, n)
    assert np.abs(Lm @ Um - A).max() / np.abs(A).max() < tol


def test_getrf_nopiv_zero_pivot():
    A = np.array([[0.0, 1.0], [1.0, 1.0]])
    S = np.ascontiguousarray(A.T)
    assert oracle.getrf_nopiv(S) == 1
    assert S[0, 1] == 1.0                      # column below the zero pivot left unscaled


def _spd(rng, n):
    G = rng.uniform(-1, 1, (n, n))
    return G @ G.T + n * np.eye(n)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [1, 5, 32, 33, 70, 130])
def test_potrf_potrs_vs_lapack(dtype, n):
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(n)
    M = _spd(rng, n)
    S = np.ascontiguousarray(M.T).astype(dtype)
    assert oracle.potrf(S) == 0
    potrf = lapack.dpotrf if dtype == np.float64 else lapack.spotrf
    c, info = potrf(M.astype(dtype), lower=1)
    assert info == 0
    eps = np.finfo(dtype).eps
    np.testing.assert_allclose(np.tril(S.T), np.tril(c), rtol=0,
                               atol=20 * eps * n * np.abs(c).max())
    b = rng.uniform(-1, 1, (2, n))
    x = oracle.potrs(S, b.astype(dtype).copy())
    xr = np.linalg.solve(M, b.T).T
    np.testing.assert_allclose(x, xr, rtol=0, atol=100 * eps * n * np.abs(xr).max())
    # unpivoted solve of the factored matrix: residual at rounding level
    r = np.abs(M @ x.astype(np.float64).T - b.T).max()
    assert r / (np.abs(M).max() * np.abs(x).max() * n * eps) < 30


@pytest.mark.parametrize("n,bad", [(5, 0), (5, 3), (70, 40), (70, 69)])
def test_potrf_failure_info_vs_lapack(n, bad):
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(n + bad)
    M = _spd(rng, n)
    M[bad, bad] = -1.0
    S = np.ascontiguousarray(M.T)
    before = S.copy()
    info = oracle.potrf(S)
    _, linfo = lapack.dpotrf(M, lower=1)
    assert info == linfo == bad + 1
    # the factorisation stops: a failure in the first panel leaves every later
    # column as it was (later failures leave them with the earlier panels' updates)
    if bad < 32:
        assert np.array_equal(S[32:], before[32:])
    # NaN on the diagonal is a failure too
    S = np.ascontiguousarray(_spd(rng, n).T)
    S[0, 0] = np.nan
    assert oracle.potrf(S) == 1


def test_oracle_dsposv_refines_and_falls_back():
    """The SPD refinement restatement: converges for kappa up to 1e6 (FP32 Cholesky +
    FP64 refinement), and an FP32 Cholesky failure (kappa 1e12) goes to the FP64
    posv with iter -3 and an accurate solution."""
    from tests.util import from_storage, scaled_residual, to_storage
    rng = np.random.default_rng(21)
    n = 80
    A = np.empty((4, n, n))
    for k, kap in enumerate([1e2, 1e4, 1e6, 1e12]):
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        M = (Q * np.geomspace(1.0, 1.0 / kap, n)) @ Q.T
        A[k] = (M + M.T) / 2
    B = rng.uniform(-1, 1, (4, n, 3))
    X, info, iters = oracle.dsposv_batched(to_storage(A), to_storage(B))
    assert np.all(info == 0)
    assert np.all(iters[:3] >= 1) and iters[0] <= iters[2], iters
    assert iters[3] == -3, iters
    assert scaled_residual(A, from_storage(X, n), B).max() <= 30


@pytest.mark.parametrize("n", [1, 7, 33, 100])
def test_oracle_getri_and_adjoint_vs_numpy(n):
    """The batched-inverse and adjoint restatements against numpy: inv(A) from the LU
    factors, and G <- A^{-T} G, GA = -(A^{-T} G) X^T from the factors of a solve."""
    rng = np.random.default_rng(200 + n)
    A = rng.uniform(-1, 1, (n, n)) + 2 * np.eye(n)
    S = np.ascontiguousarray(A.T)[None].copy()
    X = rng.uniform(-1, 1, (1, 3, n))
    ipiv, info = oracle.dgetrf_batched(S)
    assert info[0] == 0
    Inv = oracle.getri(S[0], ipiv[0])
    ref = np.linalg.inv(A)
    assert np.abs(Inv.T - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()) * n
    G = rng.standard_normal((1, 3, n))
    Gc = G.copy()
    GA = oracle.gesv_adjoint_batched(S, ipiv, X, Gc)
    gb = np.linalg.solve(A.T, G[0].T)                       # (n, 3)
    assert np.abs(Gc[0].T - gb).max() <= 1e-12 * max(1.0, np.abs(gb).max()) * n
    ga = -gb @ X[0]                                         # (n, n) = -gb x^T
    assert np.abs(GA[0].T - ga).max() <= 1e-12 * max(1.0, np.abs(ga).max()) * n
