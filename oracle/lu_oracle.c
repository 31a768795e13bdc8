/*
 * lu_oracle.c -- CPU restatement of MAGMA's batched LU factor-and-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke
 * entry and the CPU-baseline leg of the benchmark call it to verify and to
 * time against; no product code path links or calls it.
 *
 * Algorithm (right-looking, column by column, partial pivoting), restating:
 *   - LAPACK dgetf2 as called by the reference's CPU check path
 *     (testing/testing_zgesv_batched.cpp:160-176 calls lapackf77_?gesv per
 *     matrix under OpenMP): pivot = first entry of maximum magnitude in the
 *     current row order (idamax: strict '>' scan), whole-row interchange,
 *     column scaled by the reciprocal of the pivot when |pivot| >= sfmin and
 *     divided by it otherwise, rank-1 update of the trailing matrix;
 *   - MAGMA's pivot and info conventions: magmablas/zgesv_batched_small.cu:60-93
 *     (first-max scan with strict '>', zero pivot leaves the column unscaled,
 *     info = first zero-pivot column, 1-based pivots at :156) and
 *     magmablas/magma_templates.h:44-60 (ties go to the lower index);
 *   - triangular solves with the inverted diagonal multiplied in, like
 *     magmablas/trsm_template_device.cuh:53-55.
 *
 * Arithmetic contract.  Every update is one fused multiply-add
 * a = fma(-l, u, a), applied to each element in increasing elimination
 * order.  Any blocked or parallel schedule that keeps one accumulator per
 * element and applies its updates in that order (the GPU kernels do) gives
 * bit-identical factors, pivots and solutions.  Compile with
 * -ffp-contract=off so that the compiler adds no other contraction.
 *
 * Solve order (getrs):
 *   NoTrans: B <- P*B (sequential interchanges k = 0..n-1), then for
 *            t = 0..n-1: b_i = fma(-L(i,t), b_t, b_i) for i > t, then for
 *            t = n-1..0: b_t = b_t*rcp(U(t,t)) and b_i = fma(-U(i,t), b_t, b_i)
 *            for i < t.
 *   Trans:   for t = 0..n-1: b_t = b_t*rcp(U(t,t)), b_i = fma(-U(t,i), b_t, b_i)
 *            for i > t; then for t = n-1..0: b_i = fma(-L(t,i), b_t, b_i) for
 *            i < t; then interchanges in reverse order k = n-1..0 (LAPACK
 *            dgetrs with TRANS='T').
 *   rcp(u) = 1/u when |u| >= sfmin, otherwise the element is divided by u.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define DEFINE_LU(T, P, FMA, FABS, SFMIN)                                              \
                                                                                       \
/* Scale x by the reciprocal of d, or divide when d is below sfmin (LAPACK dgetf2). */ \
static inline T P##_rscale(T x, T d, T r)                                              \
{                                                                                      \
    return (FABS(d) >= SFMIN) ? x * r : x / d;                                         \
}                                                                                      \
                                                                                       \
/* First index of maximum |a| over a[0..len), strict '>' scan (idamax). */            \
static int P##_iamax(int len, const T *a, int inc)                                     \
{                                                                                      \
    int best = 0;                                                                      \
    T vmax = FABS(a[0]);                                                               \
    for (int i = 1; i < len; i++) {                                                    \
        T v = FABS(a[(size_t)i * inc]);                                                \
        if (v > vmax) { vmax = v; best = i; }                                          \
    }                                                                                  \
    return best;                                                                       \
}                                                                                      \
                                                                                       \
/* nopiv: the diagonal is the pivot (MAGMA's getrf_nopiv); ipiv may be NULL. */      \
static int P##getrf_impl(int m, int n, T *A, int lda, int *ipiv, int nopiv)            \
{                                                                                      \
    int info = 0;                                                                      \
    int mn = m < n ? m : n;                                                            \
    for (int k = 0; k < mn; k++) {                                                     \
        T *colk = A + (size_t)k * lda;                                                 \
        int p = nopiv ? k : k + P##_iamax(m - k, colk + k, 1);                         \
        if (ipiv) ipiv[k] = p + 1;                                                     \
        if (colk[p] != (T)0) {                                                         \
            if (p != k) {                                                              \
                for (int j = 0; j < n; j++) {                                          \
                    T *c = A + (size_t)j * lda;                                        \
                    T t = c[k]; c[k] = c[p]; c[p] = t;                                 \
                }                                                                      \
            }                                                                          \
            T piv = colk[k];                                                           \
            T r = (T)1 / piv;                                                          \
            for (int i = k + 1; i < m; i++) colk[i] = P##_rscale(colk[i], piv, r);     \
        } else if (info == 0) {                                                        \
            info = k + 1;                                                              \
        }                                                                              \
        for (int j = k + 1; j < n; j++) {                                              \
            T *c = A + (size_t)j * lda;                                                \
            T u = c[k];                                                                \
            for (int i = k + 1; i < m; i++) c[i] = FMA(-colk[i], u, c[i]);             \
        }                                                                              \
    }                                                                                  \
    return info;                                                                       \
}                                                                                      \
                                                                                       \
int oracle_##P##getrf(int m, int n, T *A, int lda, int *ipiv)                          \
{                                                                                      \
    return P##getrf_impl(m, n, A, lda, ipiv, 0);                                       \
}                                                                                      \
                                                                                       \
int oracle_##P##getrf_nopiv(int m, int n, T *A, int lda)                               \
{                                                                                      \
    return P##getrf_impl(m, n, A, lda, NULL, 1);                                       \
}                                                                                      \
                                                                                       \
void oracle_##P##getrs(int trans, int n, int nrhs, const T *LU, int lda,               \
                       const int *ipiv, T *B, int ldb)                                 \
{                                                                                      \
    for (int c = 0; c < nrhs; c++) {                                                   \
        T *b = B + (size_t)c * ldb;                                                    \
        if (trans == 0) {                                                              \
            for (int k = 0; k < n; k++) {                                              \
                int p = ipiv[k] - 1;                                                   \
                if (p != k) { T t = b[k]; b[k] = b[p]; b[p] = t; }                     \
            }                                                                          \
            for (int t = 0; t < n; t++) {                                              \
                const T *l = LU + (size_t)t * lda;                                     \
                for (int i = t + 1; i < n; i++) b[i] = FMA(-l[i], b[t], b[i]);         \
            }                                                                          \
            for (int t = n - 1; t >= 0; t--) {                                         \
                const T *u = LU + (size_t)t * lda;                                     \
                T d = u[t];                                                            \
                b[t] = P##_rscale(b[t], d, (T)1 / d);                                  \
                for (int i = 0; i < t; i++) b[i] = FMA(-u[i], b[t], b[i]);             \
            }                                                                          \
        } else {                                                                       \
            for (int t = 0; t < n; t++) {                                              \
                T d = LU[(size_t)t * lda + t];                                         \
                b[t] = P##_rscale(b[t], d, (T)1 / d);                                  \
                for (int i = t + 1; i < n; i++)                                        \
                    b[i] = FMA(-LU[(size_t)i * lda + t], b[t], b[i]);                  \
            }                                                                          \
            for (int t = n - 1; t >= 0; t--) {                                         \
                for (int i = 0; i < t; i++)                                            \
                    b[i] = FMA(-LU[(size_t)i * lda + t], b[t], b[i]);                  \
            }                                                                          \
            for (int k = n - 1; k >= 0; k--) {                                         \
                int p = ipiv[k] - 1;                                                   \
                if (p != k) { T t = b[k]; b[k] = b[p]; b[p] = t; }                     \
            }                                                                          \
        }                                                                              \
    }                                                                                  \
}                                                                                      \
                                                                                       \
/* Strided batch: matrix k at A + k*strideA, etc.  OpenMP over the batch with  */     \
/* dynamic scheduling, as testing/testing_zgesv_batched.cpp:160-176 does.      */     \
void oracle_##P##getrf_batched(int m, int n, T *A, int lda, long strideA,             \
                               int *ipiv, long strideP, int *info, int batch,         \
                               int nthreads)                                          \
{                                                                                      \
    (void)nthreads;                                                                    \
    _Pragma("omp parallel for schedule(dynamic) num_threads(nthreads)")               \
    for (int k = 0; k < batch; k++)                                                    \
        info[k] = oracle_##P##getrf(m, n, A + k * strideA, lda, ipiv + k * strideP);   \
}                                                                                      \
                                                                                       \
void oracle_##P##getrs_batched(int trans, int n, int nrhs, const T *A, int lda,       \
                               long strideA, const int *ipiv, long strideP,           \
                               T *B, int ldb, long strideB, int batch, int nthreads)  \
{                                                                                      \
    (void)nthreads;                                                                    \
    _Pragma("omp parallel for schedule(dynamic) num_threads(nthreads)")               \
    for (int k = 0; k < batch; k++)                                                    \
        oracle_##P##getrs(trans, n, nrhs, A + k * strideA, lda, ipiv + k * strideP,    \
                          B + k * strideB, ldb);                                       \
}                                                                                      \
                                                                                       \
void oracle_##P##gesv_batched(int n, int nrhs, T *A, int lda, long strideA,           \
                              int *ipiv, long strideP, T *B, int ldb, long strideB,   \
                              int *info, int batch, int nthreads)                     \
{                                                                                      \
    (void)nthreads;                                                                    \
    _Pragma("omp parallel for schedule(dynamic) num_threads(nthreads)")               \
    for (int k = 0; k < batch; k++) {                                                  \
        info[k] = oracle_##P##getrf(n, n, A + k * strideA, lda, ipiv + k * strideP);   \
        oracle_##P##getrs(0, n, nrhs, A + k * strideA, lda, ipiv + k * strideP,        \
                          B + k * strideB, ldb);                                       \
    }                                                                                  \
}

DEFINE_LU(double, d, fma, fabs, DBL_MIN)
DEFINE_LU(float, s, fmaf, fabsf, FLT_MIN)

/* Variable-size batch: matrix k is n[k]-by-n[k] at A + offA[k] with leading
 * dimension lda[k]; nrhs[k] right-hand sides at B + offB[k] with ldb[k]. */
void oracle_dgesv_vbatched(const int *n, const int *nrhs, double *A, const long *offA,
                           const int *lda, int *ipiv, const long *offP, double *B,
                           const long *offB, const int *ldb, int *info, int batch,
                           int nthreads)
{
    (void)nthreads;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int k = 0; k < batch; k++) {
        info[k] = oracle_dgetrf(n[k], n[k], A + offA[k], lda[k], ipiv + offP[k]);
        oracle_dgetrs(0, n[k], nrhs[k], A + offA[k], lda[k], ipiv + offP[k],
                      B + offB[k], ldb[k]);
    }
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Batched mixed-precision iterative refinement, one matrix: the restatement of
 * magma_dsgesv_gpu (src/zcgesv_gpu.cpp:144-366) in the exact arithmetic order
 * of the GPU implementation:
 *   anrm = max_i of the FP32 sum over j ascending of |(float)a_ij|; As = (float)A
 *   (overflow: iter -2);
 *   sgetrf(As) (info > 0: iter -3); X = 0, R = B;
 *   solve: X = X + (double)sgetrs(As, (float)R);
 *   residual: r_i = b_i, r_i = fma(-a_ij, x_j, r_i) for j ascending;
 *   norms: per column max|r|, max|x|; row sums over the columns (ascending);
 *   stop when every column has max|r_c| <= max|x_c| * anrm*eps*sqrt(n)
 *   (tol <= 0) or when rowmax|R| <= tol * (anrm * rowmax|X| * n * eps);
 *   checks after the initial solve (iter 0) and after each of itermax
 *   refinements; not converged: iter = -itermax-1.  When iter < 0 and
 *   fallback is set, A is overwritten by its FP64 LU and X solved in FP64.
 * Returns info. */
/* GMRES correction of the GMRES-based refinement (the GPU's
 * gm_correction_kernel; the reference's Magma_REFINE_IRGMSTRS,
 * src/dxgesv_gmres_gpu.cpp:604-780 with src/dgmres_plu_gpu.cpp): for each
 * column r of R, beta = ||r||_2 (FP64), then GMRES in FP32 on A z = r/beta,
 * right-preconditioned by the FP32 factors (sgetrs), x0 = 0, at most
 * min(n, 50) iterations, modified Gram-Schmidt, Givens rotations, stop when
 * the rotated residual |rs| <= 1e-4 (relative, rs_0 = 1) or on breakdown;
 * y from the triangular system, X += beta * sgetrs(V y).  A32 = (float)A.
 * Dot products are summed in index order (the GPU sums per thread, then
 * across threads), so the two agree to FP32 rounding, not bit for bit.
 * Returns the largest inner iteration count over the columns. */
static int gmres_correction(int n, int nrhs, const float *A32, const float *As, const int *ipiv,
                            const double *R, double *X, int ldx, double *beta_prev, int first,
                            int *stalled)
{
    const int m = n < 50 ? n : 50;
    float *V = (float *)malloc(sizeof(float) * (size_t)(m + 1) * n + 4);
    float *H = (float *)malloc(sizeof(float) * (size_t)(m + 1) * m + 4);
    float *cs = (float *)malloc(sizeof(float) * (m + 1)), *sn = (float *)malloc(sizeof(float) * (m + 1));
    float *rs = (float *)malloc(sizeof(float) * (m + 2));
    float *w = (float *)malloc(sizeof(float) * (size_t)n + 4), *z = (float *)malloc(sizeof(float) * (size_t)n + 4);
    int kmax = 0;
    /* a right-hand side whose residual 2-norm did not at least halve since the
     * previous correction ends the refinement (the GPU's GM_STALL rule) */
    *stalled = 0;
    for (int c = 0; c < nrhs; c++) {
        const double *r = R + (size_t)c * n;
        double b2 = 0.0;
        for (int i = 0; i < n; i++) b2 = fma(r[i], r[i], b2);
        const double beta = sqrt(b2);
        if (!first && !(beta <= 0.5 * beta_prev[c])) *stalled = 1;
        beta_prev[c] = beta;
    }
    if (*stalled) goto done;
    for (int c = 0; c < nrhs; c++) {
        const double *r = R + (size_t)c * n;
        const double beta = beta_prev[c];
        if (!(beta > 0.0) || isinf(beta)) continue;
        for (int i = 0; i < n; i++) V[i] = (float)(r[i] / beta);
        rs[0] = 1.0f;
        int k = 0;
        for (int it = 0; it < m; it++) {
            float *vi = V + (size_t)it * n;
            for (int i = 0; i < n; i++) z[i] = vi[i];
            oracle_sgetrs(0, n, 1, As, n, ipiv, z, n);
            for (int i = 0; i < n; i++) {
                float acc = 0.0f;
                for (int j = 0; j < n; j++) acc = fmaf(A32[i + (size_t)j * n], z[j], acc);
                w[i] = acc;
            }
            for (int j = 0; j <= it; j++) {
                const float *vj = V + (size_t)j * n;
                float h = 0.0f;
                for (int i = 0; i < n; i++) h = fmaf(w[i], vj[i], h);
                for (int i = 0; i < n; i++) w[i] = fmaf(-h, vj[i], w[i]);
                H[j * m + it] = h;
            }
            float hn2 = 0.0f;
            for (int i = 0; i < n; i++) hn2 = fmaf(w[i], w[i], hn2);
            const float hn = sqrtf(hn2);
            float *vn = V + (size_t)(it + 1) * n;
            for (int i = 0; i < n; i++) vn[i] = hn > 0.0f ? w[i] / hn : 0.0f;
            H[(it + 1) * m + it] = hn;
            for (int j = 0; j < it; j++) {
                const float t = H[j * m + it], u = H[(j + 1) * m + it];
                H[j * m + it] = cs[j] * t + sn[j] * u;
                H[(j + 1) * m + it] = -sn[j] * t + cs[j] * u;
            }
            const float a = H[it * m + it], bb = H[(it + 1) * m + it];
            float gam = hypotf(a, bb);
            if (gam == 0.0f) gam = 1e-30f;
            cs[it] = a / gam;
            sn[it] = bb / gam;
            rs[it + 1] = -sn[it] * rs[it];
            rs[it] = cs[it] * rs[it];
            H[it * m + it] = cs[it] * a + sn[it] * bb;
            k = it + 1;
            if (!(fabsf(rs[it + 1]) > 1e-4f) || bb == 0.0f) break;
        }
        for (int kk = k - 1; kk >= 0; kk--) {
            float t = rs[kk];
            for (int j = kk + 1; j < k; j++) t = fmaf(-H[kk * m + j], rs[j], t);
            rs[kk] = t / H[kk * m + kk];
        }
        for (int i = 0; i < n; i++) {
            float t = 0.0f;
            for (int j = 0; j < k; j++) t = fmaf(rs[j], V[(size_t)j * n + i], t);
            z[i] = t;
        }
        oracle_sgetrs(0, n, 1, As, n, ipiv, z, n);
        for (int i = 0; i < n; i++) X[i + (size_t)c * ldx] += beta * (double)z[i];
        if (k > kmax) kmax = k;
    }
done:
    free(V); free(H); free(cs); free(sn); free(rs); free(w); free(z);
    return kmax;
}

static int dsgesv_impl(int n, int nrhs, double *A, int lda, const double *B, int ldb, double *X,
                       int ldx, int *ipiv, int itermax, double tol, int fallback, int *iter_out,
                       int gmres, int spd);
int oracle_spotrf(int n, float *A, int lda);
void oracle_spotrs(int n, int nrhs, const float *L, int lda, float *B, int ldb);
int oracle_dpotrf(int n, double *A, int lda);
void oracle_dpotrs(int n, int nrhs, const double *L, int lda, double *B, int ldb);

/* The mixed-precision SPD refinement (the GPU's magma_dsposv_batched_work; the
 * reference's magma_dsposv_gpu, src/zcposv_gpu.cpp:134): as oracle_dsgesv with
 * the FP32 Cholesky (oracle_spotrf, lower; info > 0: iter -3) in place of the
 * FP32 LU, corrections by oracle_spotrs, and the FP64 fallback oracle_dpotrf +
 * oracle_dpotrs (the solve runs whatever the factorisation's info). */
int oracle_dsposv(int n, int nrhs, double *A, int lda, const double *B, int ldb, double *X,
                  int ldx, int itermax, double tol, int fallback, int *iter_out)
{
    return dsgesv_impl(n, nrhs, A, lda, B, ldb, X, ldx, NULL, itermax, tol, fallback, iter_out,
                       0, 1);
}

void oracle_dsposv_batched(int n, int nrhs, double *A, int lda, long strideA, const double *B,
                           int ldb, long strideB, double *X, int ldx, long strideX, int *info,
                           int *iter, int itermax, double tol, int fallback, int batch,
                           int nthreads)
{
    (void)nthreads;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int k = 0; k < batch; k++)
        info[k] = oracle_dsposv(n, nrhs, A + k * strideA, lda, B + k * strideB, ldb,
                                X + k * strideX, ldx, itermax, tol, fallback, iter + k);
}

int oracle_dsgesv(int n, int nrhs, double *A, int lda, const double *B, int ldb, double *X,
                  int ldx, int *ipiv, int itermax, double tol, int fallback, int *iter_out)
{
    return dsgesv_impl(n, nrhs, A, lda, B, ldb, X, ldx, ipiv, itermax, tol, fallback, iter_out, 0, 0);
}

/* The GMRES-based refinement (solver Magma_REFINE_IRGMSTRS): as oracle_dsgesv
 * with each correction (it >= 0; the initial solve is one sgetrs) replaced by
 * gmres_correction; iter on convergence is the total of the inner iteration
 * counts. */
int oracle_dsgesv_gmres(int n, int nrhs, double *A, int lda, const double *B, int ldb, double *X,
                        int ldx, int *ipiv, int itermax, double tol, int fallback, int *iter_out)
{
    return dsgesv_impl(n, nrhs, A, lda, B, ldb, X, ldx, ipiv, itermax, tol, fallback, iter_out, 1, 0);
}

static int dsgesv_impl(int n, int nrhs, double *A, int lda, const double *B, int ldb, double *X,
                       int ldx, int *ipiv, int itermax, double tol, int fallback, int *iter_out,
                       int gmres, int spd)
{
    const double eps = 1.1102230246251565e-16;
    double anrm = 0.0;
    int ovf = 0;
    float *As = (float *)malloc(sizeof(float) * (size_t)n * n + 4);
    float *Rs = (float *)malloc(sizeof(float) * (size_t)n * nrhs + 4);
    double *R = (double *)malloc(sizeof(double) * (size_t)n * nrhs + 8);
    for (int i = 0; i < n; i++) {
        float rs = 0.0f;             /* FP32 row sums of |float(a_ij)|, j ascending */
        for (int j = 0; j < n; j++) {
            double a = A[i + (size_t)j * lda];
            float f = (float)a;
            rs += fabsf(f);
            if (isinf(f) && !isinf(a)) ovf = 1;
            As[i + (size_t)j * n] = f;
        }
        if ((double)rs > anrm) anrm = (double)rs;
    }
    int iter = 0, info = 0, state = 0;   /* 0 active, 1 converged, 2 failed */
    int inner = 0;
    float *A32 = NULL;
    double *beta_prev = (double *)malloc(sizeof(double) * (nrhs > 0 ? nrhs : 1));
    if (gmres) {
        A32 = (float *)malloc(sizeof(float) * (size_t)n * n + 4);
        memcpy(A32, As, sizeof(float) * (size_t)n * n);
    }
    if (ovf) { iter = -2; state = 2; }
    int sinfo = spd ? oracle_spotrf(n, As, n) : oracle_sgetrf(n, n, As, n, ipiv);
    if (state == 0 && sinfo > 0) { iter = -3; state = 2; }
    for (int c = 0; c < nrhs; c++)
        for (int i = 0; i < n; i++) {
            R[i + (size_t)c * n] = B[i + (size_t)c * ldb];
            X[i + (size_t)c * ldx] = 0.0;
        }
    for (int it = -1; state == 0 && it <= itermax; it++) {
        if (it >= 0) {
            /* norms of the residual computed at the end of the previous pass */
            double rrow = 0.0, xrow = 0.0;
            int ok = 1;
            double cte = anrm * eps * sqrt((double)n);
            for (int c = 0; c < nrhs; c++) {
                double rc = 0.0, xc = 0.0;
                for (int i = 0; i < n; i++) {
                    double ra = fabs(R[i + (size_t)c * n]), xa = fabs(X[i + (size_t)c * ldx]);
                    if (ra > rc) rc = ra;
                    if (xa > xc) xc = xa;
                }
                if (!(rc <= xc * cte)) ok = 0;
            }
            for (int i = 0; i < n; i++) {
                double rs = 0.0, xs = 0.0;
                for (int c = 0; c < nrhs; c++) {
                    rs += fabs(R[i + (size_t)c * n]);
                    xs += fabs(X[i + (size_t)c * ldx]);
                }
                if (rs > rrow) rrow = rs;
                if (xs > xrow) xrow = xs;
            }
            if (tol > 0.0) ok = rrow <= tol * (anrm * xrow * (double)n * eps);
            if (ok) { state = 1; iter = gmres ? inner : it; break; }
            if (it == itermax) { state = 2; iter = -itermax - 1; break; }
        }
        if (gmres && it >= 0) {
            int stalled = 0;
            inner += gmres_correction(n, nrhs, A32, As, ipiv, R, X, ldx, beta_prev, it == 0,
                                      &stalled);
            if (stalled) { state = 2; iter = -itermax - 1; break; }
        } else {
            for (size_t e = 0; e < (size_t)n * nrhs; e++) Rs[e] = (float)R[e];
            if (spd) oracle_spotrs(n, nrhs, As, n, Rs, n);
            else oracle_sgetrs(0, n, nrhs, As, n, ipiv, Rs, n);
            for (int c = 0; c < nrhs; c++)
                for (int i = 0; i < n; i++)
                    X[i + (size_t)c * ldx] = X[i + (size_t)c * ldx] + (double)Rs[i + (size_t)c * n];
        }
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) {
                double acc = B[i + (size_t)c * ldb];
                for (int j = 0; j < n; j++)
                    acc = fma(-A[i + (size_t)j * lda], X[j + (size_t)c * ldx], acc);
                R[i + (size_t)c * n] = acc;
            }
    }
    if (state == 2 && fallback) {
        info = spd ? oracle_dpotrf(n, A, lda) : oracle_dgetrf(n, n, A, lda, ipiv);
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) X[i + (size_t)c * ldx] = B[i + (size_t)c * ldb];
        if (spd) oracle_dpotrs(n, nrhs, A, lda, X, ldx);
        else oracle_dgetrs(0, n, nrhs, A, lda, ipiv, X, ldx);
    }
    free(As); free(Rs); free(R); free(A32); free(beta_prev);
    *iter_out = iter;
    return info;
}

void oracle_dsgesv_gmres_batched(int n, int nrhs, double *A, int lda, long strideA,
                                 const double *B, int ldb, long strideB, double *X, int ldx,
                                 long strideX, int *ipiv, long strideP, int *info, int *iter,
                                 int itermax, double tol, int fallback, int batch, int nthreads)
{
    (void)nthreads;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int k = 0; k < batch; k++)
        info[k] = oracle_dsgesv_gmres(n, nrhs, A + k * strideA, lda, B + k * strideB, ldb,
                                      X + k * strideX, ldx, ipiv + k * strideP, itermax, tol,
                                      fallback, iter + k);
}

void oracle_dsgesv_batched(int n, int nrhs, double *A, int lda, long strideA, const double *B,
                           int ldb, long strideB, double *X, int ldx, long strideX, int *ipiv,
                           long strideP, int *info, int *iter, int itermax, double tol,
                           int fallback, int batch, int nthreads)
{
    (void)nthreads;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int k = 0; k < batch; k++)
        info[k] = oracle_dsgesv(n, nrhs, A + k * strideA, lda, B + k * strideB, ldb,
                                X + k * strideX, ldx, ipiv + k * strideP, itermax, tol, fallback,
                                iter + k);
}

/* Adjoint of a refinement solve (the GPU's magma_dxgesv_adjoint_*_work):
 * GB = A^{-T} G refined in FP64 with the FP32 factors of the forward call, in
 * the GPU's arithmetic order:
 *   anrm = max_j of the FP32 sum over i ascending of |(float)a_ij| (||A^T||_inf);
 *   As = (float)A factored by sgetrf (the forward's factors and pivots);
 *   GB = 0, R = G; solve: GB = GB + (double)sgetrs('T', As, (float)R);
 *   residual: r_i = g_i, r_i = fma(-a_ji, gb_j, r_i) for j ascending;
 *   norms and stopping rules of oracle_dsgesv.
 * iter_fwd < 0 (the forward fell back; A and ipiv hold FP64 factors): GB = G
 * solved by dgetrs('T') and iter = iter_fwd.  Not converged and `fallback`:
 * A and ipiv overwritten by dgetrf, GB = G solved by dgetrs('T'), the return
 * value is dgetrf's info.  Then GA = -GB X^T (acc = fma(gb_ic, x_jc, acc),
 * c ascending) when GA is not NULL. */
int oracle_dsgesv_adjoint(int n, int nrhs, double *A, int lda, int *ipiv, const double *X,
                          int ldx, const double *G, int ldg, double *GB, int ldgb, double *GA,
                          int ldga, int iter_fwd, int itermax, double tol, int fallback,
                          int *iter_out)
{
    const double eps = 1.1102230246251565e-16;
    int iter = 0, info = 0, state = 0;
    if (iter_fwd < 0) {
        state = 3;
        iter = iter_fwd;
    } else if (n > 0 && nrhs > 0) {
        float *As = (float *)malloc(sizeof(float) * (size_t)n * n + 4);
        float *Rs = (float *)malloc(sizeof(float) * (size_t)n * nrhs + 4);
        double *R = (double *)malloc(sizeof(double) * (size_t)n * nrhs + 8);
        int *ps = (int *)malloc(sizeof(int) * (size_t)n + 4);
        double anrm = 0.0;
        for (int j = 0; j < n; j++) {
            float cs = 0.0f;
            for (int i = 0; i < n; i++) {
                float f = (float)A[i + (size_t)j * lda];
                cs += fabsf(f);
                As[i + (size_t)j * n] = f;
            }
            if ((double)cs > anrm) anrm = (double)cs;
        }
        oracle_sgetrf(n, n, As, n, ps);
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) {
                R[i + (size_t)c * n] = G[i + (size_t)c * ldg];
                GB[i + (size_t)c * ldgb] = 0.0;
            }
        for (int it = -1; state == 0 && it <= itermax; it++) {
            if (it >= 0) {
                double rrow = 0.0, xrow = 0.0;
                int ok = 1;
                double cte = anrm * eps * sqrt((double)n);
                for (int c = 0; c < nrhs; c++) {
                    double rc = 0.0, xc = 0.0;
                    for (int i = 0; i < n; i++) {
                        double ra = fabs(R[i + (size_t)c * n]), xa = fabs(GB[i + (size_t)c * ldgb]);
                        if (ra > rc) rc = ra;
                        if (xa > xc) xc = xa;
                    }
                    if (!(rc <= xc * cte)) ok = 0;
                }
                for (int i = 0; i < n; i++) {
                    double rs = 0.0, xs = 0.0;
                    for (int c = 0; c < nrhs; c++) {
                        rs += fabs(R[i + (size_t)c * n]);
                        xs += fabs(GB[i + (size_t)c * ldgb]);
                    }
                    if (rs > rrow) rrow = rs;
                    if (xs > xrow) xrow = xs;
                }
                if (tol > 0.0) ok = rrow <= tol * (anrm * xrow * (double)n * eps);
                if (ok) { state = 1; iter = it; break; }
                if (it == itermax) { state = 2; iter = -itermax - 1; break; }
            }
            for (size_t e = 0; e < (size_t)n * nrhs; e++) Rs[e] = (float)R[e];
            oracle_sgetrs(1, n, nrhs, As, n, ps, Rs, n);
            for (int c = 0; c < nrhs; c++)
                for (int i = 0; i < n; i++)
                    GB[i + (size_t)c * ldgb] = GB[i + (size_t)c * ldgb] + (double)Rs[i + (size_t)c * n];
            for (int c = 0; c < nrhs; c++)
                for (int i = 0; i < n; i++) {
                    double acc = G[i + (size_t)c * ldg];
                    for (int j = 0; j < n; j++)
                        acc = fma(-A[j + (size_t)i * lda], GB[j + (size_t)c * ldgb], acc);
                    R[i + (size_t)c * n] = acc;
                }
        }
        free(As); free(Rs); free(R); free(ps);
    }
    if (state == 2 && fallback) {
        info = oracle_dgetrf(n, n, A, lda, ipiv);
        state = 3;
    }
    if (state == 3) {
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) GB[i + (size_t)c * ldgb] = G[i + (size_t)c * ldg];
        oracle_dgetrs(1, n, nrhs, A, lda, ipiv, GB, ldgb);
    }
    if (GA)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                double acc = 0.0;
                for (int c = 0; c < nrhs; c++)
                    acc = fma(GB[i + (size_t)c * ldgb], X[j + (size_t)c * ldx], acc);
                GA[i + (size_t)j * ldga] = -acc;
            }
    *iter_out = iter;
    return info;
}

/* Adjoint of x = A^{-1} b with the forward LU kept: G <- A^{-T} G (getrs with
 * TRANS='T'), then GA(i,j) = -(sum_c G(i,c) X(j,c)) accumulated as
 * acc = fma(G(i,c), X(j,c), acc) for c ascending from acc = 0. */
#define DEFINE_ADJOINT(T, P, FMA)                                                          \
void oracle_##P##gesv_adjoint(int n, int nrhs, const T *LU, int lda, const int *ipiv,    \
                              const T *X, int ldx, T *G, int ldg, T *GA, int ldga)       \
{                                                                                        \
    oracle_##P##getrs(1, n, nrhs, LU, lda, ipiv, G, ldg);                                \
    for (int j = 0; j < n; j++)                                                          \
        for (int i = 0; i < n; i++) {                                                    \
            T acc = (T)0;                                                                \
            for (int c = 0; c < nrhs; c++)                                               \
                acc = FMA(G[i + (size_t)c * ldg], X[j + (size_t)c * ldx], acc);          \
            GA[i + (size_t)j * ldga] = -acc;                                             \
        }                                                                                \
}                                                                                        \
void oracle_##P##gesv_adjoint_batched(int n, int nrhs, const T *LU, int lda, long sLU,   \
                                      const int *ipiv, long sP, const T *X, int ldx,     \
                                      long sX, T *G, int ldg, long sG, T *GA, int ldga,  \
                                      long sGA, int batch, int nthreads)                 \
{                                                                                        \
    (void)nthreads;                                                                      \
    _Pragma("omp parallel for schedule(dynamic) num_threads(nthreads)")                 \
    for (int k = 0; k < batch; k++)                                                      \
        oracle_##P##gesv_adjoint(n, nrhs, LU + k * sLU, lda, ipiv + k * sP, X + k * sX,  \
                                 ldx, G + k * sG, ldg, GA + k * sGA, ldga);              \
}
DEFINE_ADJOINT(double, d, fma)
DEFINE_ADJOINT(float, s, fmaf)

/* Random butterfly transformation, the GPU's arithmetic (magma_gb300/csrc
 * rbt.cu, restating the depth-2 RBT of the reference's magma_dgerbt_batched):
 * level 0 is one butterfly of order n, level 1 two of orders ceil(n/2) and
 * n - ceil(n/2); a block of order m pairs (i, i + m/2), the last index of an
 * odd block is unpaired; R = w[base + k], S = w[base + k + m/2] with base 0
 * (level 0) or n + block start (level 1); c = 1/sqrt 2. */
static const double RBT_C = 0.70710678118654752440;

static void rbt_block(int level, int n, int x, int *b0, int *g)
{
    if (level == 0) { *b0 = 0; *g = n / 2; return; }
    int n1 = (n + 1) / 2;
    if (x < n1) { *b0 = 0; *g = n1 / 2; } else { *b0 = n1; *g = (n - n1) / 2; }
}

/* A <- U^T A V one level at a time (inner, then outer); per 2x2 group the
 * column transform first, then the row transform. */
void oracle_rbt_matrix(int n, double *A, int lda, const double *u, const double *v)
{
    for (int level = 1; level >= 0; level--) {
        for (int ri = 0; ri < n; ri++) {
            int rb0, rg;
            rbt_block(level, n, ri, &rb0, &rg);
            int ki = ri - rb0;
            if (ki >= rg && ki != 2 * rg) continue;      /* bottoms are handled with their tops */
            int rpair = ki < rg, ri2 = ri + rg;
            for (int cj = 0; cj < n; cj++) {
                int cb0, cg;
                rbt_block(level, n, cj, &cb0, &cg);
                int kj = cj - cb0;
                if (kj >= cg && kj != 2 * cg) continue;
                int cpair = kj < cg, cj2 = cj + cg;
                double a = A[ri + (size_t)cj * lda];
                double b = cpair ? A[ri + (size_t)cj2 * lda] : 0.0;
                double c = rpair ? A[ri2 + (size_t)cj * lda] : 0.0;
                double d = (rpair && cpair) ? A[ri2 + (size_t)cj2 * lda] : 0.0;
                if (cpair) {
                    int vb = (level == 0 ? 0 : n + cb0) + kj;
                    double wr = RBT_C * v[vb], ws = RBT_C * v[vb + cg];
                    double a1 = wr * (a + b), b1 = ws * (a - b);
                    double c1 = wr * (c + d), d1 = ws * (c - d);
                    a = a1; b = b1; c = c1; d = d1;
                }
                if (rpair) {
                    int ub = (level == 0 ? 0 : n + rb0) + ki;
                    double wr = RBT_C * u[ub], ws = RBT_C * u[ub + rg];
                    double a1 = wr * (a + c), c1 = ws * (a - c);
                    double b1 = wr * (b + d), d1 = ws * (b - d);
                    a = a1; c = c1; b = b1; d = d1;
                }
                A[ri + (size_t)cj * lda] = a;
                if (cpair) A[ri + (size_t)cj2 * lda] = b;
                if (rpair) A[ri2 + (size_t)cj * lda] = c;
                if (rpair && cpair) A[ri2 + (size_t)cj2 * lda] = d;
            }
        }
    }
}

/* trans: B <- U^T B (inner level, then outer); else B <- V B (outer, then
 * inner). */
void oracle_rbt_vectors(int trans, int n, int nrhs, const double *w, double *B, int ldb)
{
    for (int step = 0; step < 2; step++) {
        int level = trans ? 1 - step : step;
        for (int col = 0; col < nrhs; col++) {
            double *x = B + (size_t)col * ldb;
            for (int ri = 0; ri < n; ri++) {
                int b0, g;
                rbt_block(level, n, ri, &b0, &g);
                int k = ri - b0;
                if (k >= g) continue;
                int wb = (level == 0 ? 0 : n + b0) + k;
                double R = w[wb], S = w[wb + g];
                double xt = x[ri], yb = x[ri + g];
                if (trans) {
                    x[ri] = (RBT_C * R) * (xt + yb);
                    x[ri + g] = (RBT_C * S) * (xt - yb);
                } else {
                    double p = R * xt, q = S * yb;
                    x[ri] = RBT_C * (p + q);
                    x[ri + g] = RBT_C * (p - q);
                }
            }
        }
    }
}

/* Cholesky A = L L^T (lower) and its solve, the GPU's order (magma_gb300/csrc
 * chol.cu; the reference's magma_?potrf_batched / potrs / posv): 32-column
 * panels; per panel the diagonal block right-looking (l_kk = sqrt(a_kk),
 * column below scaled by 1/l_kk with the sfmin rule, a_it = fma(-l_ik, l_tk,
 * a_it) for i >= t > k), then every row below solved against L11 (k
 * ascending), then A22 -= L21 L21^T on the lower triangle (k ascending).  A
 * pivot that is not > 0 (or NaN) at column j returns info = j + 1 at once,
 * the diagonal block left as updated so far.  Solve: L y = b then L^T x = y,
 * each with the diagonal multiplied in as a reciprocal. */
#define DEFINE_CHOL(T, P, FMA, SQRT)                                                        \
int oracle_##P##potrf(int n, T *A, int lda)                                                 \
{                                                                                           \
    for (int j0 = 0; j0 < n; j0 += 32) {                                                    \
        int ib = n - j0 < 32 ? n - j0 : 32;                                                 \
        for (int k = 0; k < ib; k++) {                                                      \
            T d = A[(j0 + k) + (size_t)(j0 + k) * lda];                                     \
            if (!(d > (T)0)) return j0 + k + 1;                                             \
            T s = SQRT(d), r = (T)1 / s;                                                    \
            A[(j0 + k) + (size_t)(j0 + k) * lda] = s;                                       \
            for (int i = k + 1; i < ib; i++) {                                              \
                T *x = &A[(j0 + i) + (size_t)(j0 + k) * lda];                               \
                *x = P##_rscale(*x, s, r);                                                  \
            }                                                                               \
            for (int t = k + 1; t < ib; t++) {                                              \
                T ltk = A[(j0 + t) + (size_t)(j0 + k) * lda];                               \
                for (int i = t; i < ib; i++) {                                              \
                    T *x = &A[(j0 + i) + (size_t)(j0 + t) * lda];                           \
                    *x = FMA(-A[(j0 + i) + (size_t)(j0 + k) * lda], ltk, *x);               \
                }                                                                           \
            }                                                                               \
        }                                                                                   \
        for (int i = j0 + ib; i < n; i++)                                                   \
            for (int k = 0; k < ib; k++) {                                                  \
                T lkk = A[(j0 + k) + (size_t)(j0 + k) * lda];                               \
                T *xk = &A[i + (size_t)(j0 + k) * lda];                                     \
                *xk = P##_rscale(*xk, lkk, (T)1 / lkk);                                     \
                for (int t = k + 1; t < ib; t++) {                                          \
                    T *xt = &A[i + (size_t)(j0 + t) * lda];                                 \
                    *xt = FMA(-*xk, A[(j0 + t) + (size_t)(j0 + k) * lda], *xt);             \
                }                                                                           \
            }                                                                               \
        for (int c = j0 + ib; c < n; c++)                                                   \
            for (int r = c; r < n; r++) {                                                   \
                T acc = A[r + (size_t)c * lda];                                             \
                for (int k = 0; k < ib; k++)                                                \
                    acc = FMA(-A[r + (size_t)(j0 + k) * lda], A[c + (size_t)(j0 + k) * lda], \
                              acc);                                                         \
                A[r + (size_t)c * lda] = acc;                                               \
            }                                                                               \
    }                                                                                       \
    return 0;                                                                               \
}                                                                                           \
                                                                                            \
void oracle_##P##potrs(int n, int nrhs, const T *L, int lda, T *B, int ldb)                 \
{                                                                                           \
    for (int c = 0; c < nrhs; c++) {                                                        \
        T *b = B + (size_t)c * ldb;                                                         \
        for (int t = 0; t < n; t++) {                                                       \
            T d = L[t + (size_t)t * lda];                                                   \
            b[t] = P##_rscale(b[t], d, (T)1 / d);                                           \
            for (int i = t + 1; i < n; i++) b[i] = FMA(-L[i + (size_t)t * lda], b[t], b[i]); \
        }                                                                                   \
        for (int t = n - 1; t >= 0; t--) {                                                  \
            T d = L[t + (size_t)t * lda];                                                   \
            b[t] = P##_rscale(b[t], d, (T)1 / d);                                           \
            for (int i = 0; i < t; i++) b[i] = FMA(-L[t + (size_t)i * lda], b[t], b[i]);    \
        }                                                                                   \
    }                                                                                       \
}
DEFINE_CHOL(double, d, fma, sqrt)
DEFINE_CHOL(float, s, fmaf, sqrtf)
