"""The interchange algebra the blocked factorisation's kernels rely on, checked on
the host against LAPACK's sequential application of the pivots.

* band_kernel resolves, for each lane, where the content of top row j0+k and of
  pivot row p_k comes from after the step's interchanges k = 0..ib-1, by
  running the transpositions from the last to the first; a row below the top
  block only ever receives an original top row.
* left_swaps_kernel applies, after the last step, the interchanges of all later
  panels to an earlier panel's columns as one gather new[i] = old[tau(i)],
  tau = P_pj1 o ... o P_mn-1, each row resolved independently the same way.
* the oracle's GMRES-based refinement converges where it should, ends stalled
  refinement, and falls back to FP64."""
import numpy as np
import pytest

import oracle
from tests.util import from_storage, scaled_residual, to_storage


def _apply_sequential(rows, pivots, start):
    """LAPACK order: for k = start.. swap rows k and pivots[k - start] (0-based)."""
    x = list(rows)
    for k, p in enumerate(pivots, start):
        x[k], x[p] = x[p], x[k]
    return x


def _tau(i, pivots, start):
    """Source row of row i after the interchanges, transpositions run backwards."""
    v = i
    for k in range(start + len(pivots) - 1, start - 1, -1):
        p = pivots[k - start]
        if v == k:
            v = p
        elif v == p:
            v = k
    return v


def _random_pivots(rng, m, j0, ib):
    return [int(rng.integers(k, m)) for k in range(j0, j0 + ib)]


@pytest.mark.parametrize("seed", range(20))
def test_step_resolution_matches_sequential_interchanges(seed):
    rng = np.random.default_rng(seed)
    m, j0 = int(rng.integers(40, 300)), int(rng.integers(0, 8)) * 32
    m = max(m, j0 + 33)
    ib = min(32, m - j0)
    piv = _random_pivots(rng, m, j0, ib)
    seq = _apply_sequential(range(m), piv, j0)
    for i in range(m):
        assert seq[i] == _tau(i, piv, j0)
    top = set(range(j0, j0 + ib))
    for i in range(j0 + ib, m):
        if seq[i] != i:
            assert seq[i] in top          # rows below receive original top rows only
    # the top rows' sources, resolved per lane, with the pivot index of a source below
    for k in range(ib):
        v, idx = j0 + k, -1
        for kk in range(ib - 1, -1, -1):
            a, p = j0 + kk, piv[kk]
            if v == a:
                v, idx = p, kk
            elif v == p:
                v, idx = a, -1
        assert v == seq[j0 + k]
        if v >= j0 + ib:
            assert idx >= 0 and piv[idx] == v


@pytest.mark.parametrize("seed", range(10))
def test_deferred_left_interchanges_equal_stepwise(seed):
    """Applying each panel's interchanges to the earlier panels step by step (LAPACK)
    equals one gather per earlier panel after the last step."""
    rng = np.random.default_rng(100 + seed)
    m = int(rng.integers(33, 260))
    n = int(rng.integers(33, 260))
    mn = min(m, n)
    widths, j = [], 0
    while j < mn:
        w = min(int(rng.choice([8, 16, 32])), mn - j)
        widths.append(w)
        j += w
    piv = [int(rng.integers(k, m)) for k in range(mn)]
    starts = np.cumsum([0] + widths[:-1])
    A = rng.standard_normal((m, mn))
    step = A.copy()
    for b, (j0, w) in enumerate(zip(starts, widths)):
        for k in range(j0, j0 + w):                  # this panel's interchanges on the columns to its left
            p = piv[k]
            step[[k, p], :j0] = step[[p, k], :j0]
    deferred = A.copy()
    for b, (pj0, w) in enumerate(zip(starts, widths)):
        pj1 = pj0 + w
        if pj1 >= mn:
            continue
        later = piv[pj1:mn]
        src = [_tau(i, later, pj1) for i in range(pj1, m)]
        deferred[pj1:, pj0:pj1] = A[src, pj0:pj1]
    assert np.array_equal(step, deferred)


def test_oracle_gmres_refinement_converges_stalls_and_falls_back():
    from magma_gb300.testing import svd_batch_torch
    n = 64
    A = svd_batch_torch(4, n, [1e2, 1e4, 1e6, 1e13], 11, device="cpu").numpy()
    Bm = np.random.default_rng(11).uniform(-1, 1, (4, n, 2))
    S, B = to_storage(A), to_storage(Bm)
    X, ipiv, info, iters = oracle.dsgesv_gmres_batched(S.copy(), B, itermax=10)
    assert np.all(info == 0)
    assert np.all(iters[:3] >= 0), iters              # converged: total inner iterations
    assert iters[0] <= iters[2]
    assert iters[3] == -11, iters                     # stalled or not converged: FP64 re-solve
    assert scaled_residual(A, from_storage(X, n), Bm).max() <= 30
    Xn, _, _, itn = oracle.dsgesv_gmres_batched(S.copy(), B, itermax=10, fallback=False)
    assert itn[3] == -11
    assert scaled_residual(A[:3], from_storage(Xn[:3], n), Bm[:3]).max() <= 30
