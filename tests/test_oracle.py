"""Pin the CPU oracle against LAPACK's own outputs (tests/golden/lapack_golden.npz).

The reference's CPU path is LAPACK ?getrf/?getrs per matrix
(testing/testing_zgesv_batched.cpp:160-176); its acceptance criteria are the
scaled residual < 30 (testing/magma_util.cpp:138,192), ||PA-LU|| < 30 eps and
an exact pivot match reported by --check2 (testing_zgetrf_batched.cpp:86-111).
The oracle must meet all three against LAPACK: identical info, identical
pivots except where the two candidates are a near-tie, factors and solutions
equal to rounding.
"""
import numpy as np
import pytest

import oracle
from tests.util import EPS, explain_pivot_mismatch, from_storage, lu_error, scaled_residual, to_storage

GOLDEN_CASES = None


def _cases(golden):
    return sorted({k.split("/")[0] for k in golden.files if not k.startswith("meta")})


def pytest_generate_tests(metafunc):
    if "case" in metafunc.fixturenames:
        import numpy as _np
        from pathlib import Path
        g = _np.load(Path(__file__).parent / "golden" / "lapack_golden.npz")
        metafunc.parametrize("case", _cases(g))


def test_oracle_builds():
    assert oracle.load() is not None
    assert oracle.max_threads() >= 1


def test_oracle_vs_lapack(golden, case):
    A = golden[f"{case}/A"]
    dt = A.dtype.type
    eps = EPS[dt]
    b, m, n = A.shape
    S = to_storage(A)
    getrf = oracle.dgetrf_batched if dt == np.float64 else oracle.sgetrf_batched
    ipiv, info = getrf(S, m)
    np.testing.assert_array_equal(info, golden[f"{case}/info"])
    ref_piv = golden[f"{case}/ipiv"]
    LU = from_storage(S, m)
    for k in range(b):
        why = explain_pivot_mismatch(A[k], ref_piv[k], ipiv[k])
        if why is not None:
            step, gap = why
            assert gap < 1e3 * eps, f"{case}[{k}] pivot mismatch at step {step}, rel gap {gap:g}"
    # backward error of the oracle's own factors, the reference's getrf check
    err = lu_error(A, LU, ipiv)
    assert np.all(err < 30 * eps), err
    # factors equal LAPACK's to rounding where the pivots agree
    same = np.all(ref_piv == ipiv, axis=1)
    if same.any():
        d = np.abs(LU[same].astype(np.float64) - golden[f"{case}/LU"][same].astype(np.float64))
        scale = np.abs(golden[f"{case}/LU"][same]).max() + 1.0
        assert d.max() <= 1e3 * n * eps * scale
    if f"{case}/B" in golden.files and info.max() == 0:
        B = golden[f"{case}/B"]
        getrs = oracle.dgetrs_batched if dt == np.float64 else oracle.sgetrs_batched
        for trans, key in ((False, "XN"), (True, "XT")):
            X = to_storage(B)
            getrs(S, ipiv, X, trans=trans)
            Xm = from_storage(X, n)
            Aop = np.transpose(A, (0, 2, 1)) if trans else A
            res = scaled_residual(Aop, Xm, B) * (EPS[np.float64] / eps)
            assert np.all(res < 30), (case, trans, res.max())
            if same.all():
                ref = golden[f"{case}/{key}"]
                rel = np.abs(Xm - ref).max() / (np.abs(ref).max() + 1e-300)
                assert rel < 1e6 * eps, (case, trans, rel)


def test_oracle_gesv_equals_getrf_getrs():
    rng = np.random.default_rng(7)
    A = rng.uniform(-1, 1, size=(17, 20, 20))
    B = rng.uniform(-1, 1, size=(17, 20, 3))
    S1, X1 = to_storage(A), to_storage(B)
    ipiv1, info1 = oracle.dgesv_batched(S1, X1)
    S2, X2 = to_storage(A), to_storage(B)
    ipiv2, info2 = oracle.dgetrf_batched(S2)
    oracle.dgetrs_batched(S2, ipiv2, X2)
    assert np.array_equal(S1, S2) and np.array_equal(X1, X2) and np.array_equal(ipiv1, ipiv2)


def test_oracle_zero_pivot_semantics():
    """info = first zero column (1-based); the factorisation continues past it."""
    A = np.array([[[0.0, 1.0, 2.0], [0.0, 3.0, 4.0], [0.0, 5.0, 7.0]]])
    S = to_storage(A)
    ipiv, info = oracle.dgetrf_batched(S)
    assert info[0] == 1
    assert ipiv[0, 0] == 1                      # no interchange on a zero column
    LU = from_storage(S, 3)
    assert LU[0, 1, 1] == 5.0                   # next column still pivoted and factored


def test_oracle_nan_pivot_follows_idamax():
    """A NaN at the diagonal is chosen (strict '>' scan never replaces it); a NaN
    below the diagonal is never chosen."""
    A = np.array([[[np.nan, 1.0], [2.0, 3.0]], [[1.0, 1.0], [np.nan, 3.0]]])
    S = to_storage(A)
    ipiv, _ = oracle.dgetrf_batched(S)
    assert ipiv[0, 0] == 1 and ipiv[1, 0] == 1


def test_oracle_ties_go_to_first_row():
    A = np.array([[[1.0, 2.0, 0.0], [-1.0, 1.0, 1.0], [1.0, 0.0, 3.0]]])
    S = to_storage(A)
    ipiv, _ = oracle.dgetrf_batched(S)
    assert ipiv[0, 0] == 1


def test_oracle_vbatched_matches_fixed():
    rng = np.random.default_rng(11)
    ns = [5, 17, 33, 1]
    As = [rng.uniform(-1, 1, size=(n, n)) for n in ns]
    Bs = [rng.uniform(-1, 1, size=(n, 2)) for n in ns]
    Sv = [a.T.copy() for a in As]
    Xv = [b.T.copy() for b in Bs]
    pivs, info = oracle.dgesv_vbatched(ns, [2] * 4, Sv, Xv)
    for k, n in enumerate(ns):
        S = to_storage(As[k][None])
        X = to_storage(Bs[k][None])
        p, i = oracle.dgesv_batched(S, X)
        assert np.array_equal(S[0], Sv[k]) and np.array_equal(X[0], Xv[k])
        assert np.array_equal(p[0], pivs[k])
