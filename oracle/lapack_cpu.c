/* lapack_cpu.c -- the reference's CPU path for batched LU solves, timed as the
 * CPU baseline of the benchmark.  Benchmark and test infrastructure only: the
 * library never loads it.
 *
 * MAGMA's batched gesv tester checks the GPU against LAPACK on the host: one
 * dgesv (dgetrf + dgetrs) per matrix, the batch spread over OpenMP threads with
 * schedule(dynamic) and the BLAS kept single-threaded inside each call
 * (testing/testing_zgesv_batched.cpp:160-176, magma_set_lapack_numthreads(1)).
 * This file does the same against the LAPACK that scipy bundles (OpenBLAS, its
 * symbols prefixed scipy_), opened at run time with dlopen, so it needs no
 * link-time BLAS.  The adjoint form adds dgetrs('T') for the transposed solve
 * and dger for the rank-nrhs outer product gA = -gb x^T.
 *
 * Matrices are reached through arrays of host pointers (one per matrix), with
 * per-matrix order, right-hand sides and leading dimensions, so one entry
 * serves uniform and variable-size batches.
 */
#include <dlfcn.h>
#include <omp.h>
#include <stdlib.h>

typedef void (*gesv_t)(const int *, const int *, double *, const int *, int *, double *, const int *,
                       int *);
typedef void (*getrf_t)(const int *, const int *, double *, const int *, int *, int *);
typedef void (*getrs_t)(const char *, const int *, const int *, const double *, const int *,
                        const int *, double *, const int *, int *, size_t);
typedef void (*ger_t)(const int *, const int *, const double *, const double *, const int *,
                      const double *, const int *, double *, const int *);
typedef void (*setnt_t)(int);

static gesv_t p_dgesv;
static getrf_t p_dgetrf;
static getrs_t p_dgetrs;
static ger_t p_dger;

/* Opens the LAPACK library at `path`; 0 on success, -1 when it or one of its
 * symbols is missing. */
int lapack_open(const char *path)
{
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    p_dgesv = (gesv_t)dlsym(h, "scipy_dgesv_");
    p_dgetrf = (getrf_t)dlsym(h, "scipy_dgetrf_");
    p_dgetrs = (getrs_t)dlsym(h, "scipy_dgetrs_");
    p_dger = (ger_t)dlsym(h, "scipy_dger_");
    setnt_t setnt = (setnt_t)dlsym(h, "scipy_openblas_set_num_threads");
    if (!p_dgesv || !p_dgetrf || !p_dgetrs || !p_dger || !setnt) return -1;
    setnt(1); /* one BLAS thread per call, the tester's magma_set_lapack_numthreads(1) */
    return 0;
}

int lapack_max_threads(void) { return omp_get_max_threads(); }

/* Per matrix k, the tester's lapackf77_dgesv: A_k = P L U, B_k := A_k^{-1} B_k
 * (dgetrf then dgetrs inside LAPACK's dgesv); info[k] from it. */
void lapack_dgesv_ptrs(int batch, const int *n, const int *nrhs, double **A, const int *lda,
                       double **B, const int *ldb, int *info, int max_n, int nthreads)
{
#pragma omp parallel num_threads(nthreads)
    {
        int *ipiv = (int *)malloc(sizeof(int) * (size_t)(max_n > 0 ? max_n : 1));
#pragma omp for schedule(dynamic)
        for (int k = 0; k < batch; k++) {
            int inf = 0;
            p_dgesv(&n[k], &nrhs[k], A[k], &lda[k], ipiv, B[k], &ldb[k], &inf);
            info[k] = inf;
        }
        free(ipiv);
    }
}

/* Forward and adjoint solve per matrix: dgetrf, X = A^{-1} B (B overwritten),
 * GB = A^{-T} G (G overwritten), GA = -GB X^T (GA n x n, leading dimension lda). */
void lapack_dgesv_adjoint_ptrs(int batch, const int *n, const int *nrhs, double **A, const int *lda,
                               double **B, const int *ldb, double **G, double **GA, int *info,
                               int max_n, int nthreads)
{
#pragma omp parallel num_threads(nthreads)
    {
        int *ipiv = (int *)malloc(sizeof(int) * (size_t)(max_n > 0 ? max_n : 1));
        const double minus_one = -1.0;
        const int one = 1;
#pragma omp for schedule(dynamic)
        for (int k = 0; k < batch; k++) {
            int inf = 0, inf2 = 0;
            p_dgetrf(&n[k], &n[k], A[k], &lda[k], ipiv, &inf);
            info[k] = inf;
            if (inf != 0) continue;
            p_dgetrs("N", &n[k], &nrhs[k], A[k], &lda[k], ipiv, B[k], &ldb[k], &inf2, 1);
            p_dgetrs("T", &n[k], &nrhs[k], A[k], &lda[k], ipiv, G[k], &ldb[k], &inf2, 1);
            for (size_t e = 0; e < (size_t)lda[k] * n[k]; e++) GA[k][e] = 0.0;
            for (int c = 0; c < nrhs[k]; c++)
                p_dger(&n[k], &n[k], &minus_one, G[k] + (size_t)c * ldb[k], &one,
                       B[k] + (size_t)c * ldb[k], &one, GA[k], &lda[k]);
        }
        free(ipiv);
    }
}
