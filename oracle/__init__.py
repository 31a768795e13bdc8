"""CPU oracle for the batched LU path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, as the checker and as the timed CPU reference; the product path never
imports it.  See lu_oracle.c for the algorithm and the reference lines it
restates; lapack_cpu.c (oracle.lapack) is the reference tester's own CPU path
(LAPACK dgesv per matrix, through scipy's bundled OpenBLAS), timed as the CPU
baseline.  The restatement is pinned against LAPACK (the library the
reference's CPU check path calls) by the golden fixtures in tests/golden/.
"""
from .oracle import (build, dgesv_batched, dsgesv_adjoint, dsgesv_batched, dsgesv_gmres_batched, dsgesv_vbatched, dsposv_batched, gesv_adjoint_batched, dgetrf, dgetrf_batched, dgetrs, dgetrs_batched, getrf_nopiv, getri, potrf, potrs, rbt_matrix, rbt_vectors,  # noqa: F401
                     dgesv_vbatched, load, max_threads, sgesv_batched, sgesv_vbatched, sgetrf,
                     sgetrf_batched, sgetrs, sgetrs_batched)
