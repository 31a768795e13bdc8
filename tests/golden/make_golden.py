"""Generate the LAPACK golden vectors that pin the CPU oracle.

The reference's CPU check path (testing/testing_zgesv_batched.cpp:160-176,
testing/testing_zgetrf_batched.cpp:86-111) calls LAPACK ?getrf/?getrs per
matrix.  This script runs LAPACK itself -- scipy's bundled OpenBLAS build,
through scipy.linalg.lapack -- on seeded inputs and stores inputs and outputs
in lapack_golden.npz.  Run it from the repository root:

    python tests/golden/make_golden.py

Cases (each a small batch of column-major matrices):
  uniform_n{n}   entries uniform(-1,1) (larnv idist=2 style), nrhs=3
  singular_n{n}  uniform with columns 1 and n//2 zeroed (the reference's
                 SINGULARITY_CHECK, testing/testing_zgetrf_batched.cpp:33-40)
  ties_n{n}      small integers, so that pivot candidates tie exactly
  rect_{m}x{n}   rectangular getrf
Float32 cases carry the prefix s_.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import scipy
import scipy.linalg.lapack as lp

OUT = Path(__file__).resolve().parent / "lapack_golden.npz"


def lapack_case(A, B, dtype):
    """A: (batch, m, n) math orientation; B: (batch, n, nrhs) or None."""
    getrf = lp.dgetrf if dtype == np.float64 else lp.sgetrf
    getrs = lp.dgetrs if dtype == np.float64 else lp.sgetrs
    b = A.shape[0]
    LU, P, INFO, XN, XT = [], [], [], [], []
    for k in range(b):
        lu, piv, info = getrf(A[k].astype(dtype), overwrite_a=False)
        LU.append(lu)
        P.append(piv + 1)                       # scipy returns 0-based pivots
        INFO.append(info)
        if B is not None and A.shape[1] == A.shape[2]:
            xn, inf1 = getrs(lu, piv, B[k].astype(dtype), trans=0)
            xt, inf2 = getrs(lu, piv, B[k].astype(dtype), trans=1)
            XN.append(xn)
            XT.append(xt)
    out = {"A": A.astype(dtype), "LU": np.stack(LU), "ipiv": np.stack(P).astype(np.int32),
           "info": np.array(INFO, dtype=np.int32)}
    if XN:
        out["B"] = B.astype(dtype)
        out["XN"] = np.stack(XN)
        out["XT"] = np.stack(XT)
    return out


def main():
    rng = np.random.default_rng(20240601)
    cases = {}
    for dt, pre in ((np.float64, ""), (np.float32, "s_")):
        sizes = (1, 2, 3, 5, 8, 16, 31, 32, 33, 48, 64, 100) if pre == "" else (1, 2, 5, 16, 32, 33, 64)
        for n in sizes:
            bsz = 6 if n <= 16 else (4 if n <= 48 else 2)
            A = rng.uniform(-1, 1, size=(bsz, n, n))
            B = rng.uniform(-1, 1, size=(bsz, n, 3))
            cases[f"{pre}uniform_n{n}"] = lapack_case(A, B, dt)
        for n in (4, 16, 32, 40):
            A = rng.uniform(-1, 1, size=(3, n, n))
            A[:, :, 1] = 0.0
            A[:, :, n // 2] = 0.0
            B = rng.uniform(-1, 1, size=(3, n, 2))
            cases[f"{pre}singular_n{n}"] = lapack_case(A, B, dt)
        for n in (3, 6, 12, 24, 32):
            A = rng.integers(-2, 3, size=(6, n, n)).astype(np.float64)
            B = rng.integers(-2, 3, size=(6, n, 2)).astype(np.float64)
            cases[f"{pre}ties_n{n}"] = lapack_case(A, B, dt)
        for m, n in ((40, 24), (24, 40), (70, 33), (33, 70)):
            A = rng.uniform(-1, 1, size=(3, m, n))
            cases[f"{pre}rect_{m}x{n}"] = lapack_case(A, None, dt)
    flat = {}
    for name, d in cases.items():
        for key, v in d.items():
            flat[f"{name}/{key}"] = v
    flat["meta/lapack"] = np.array(f"scipy {scipy.__version__} LAPACK (bundled OpenBLAS)")
    np.savez_compressed(OUT, **flat)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(cases)} cases)")


if __name__ == "__main__":
    sys.exit(main())
