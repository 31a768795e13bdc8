// ir.cu -- batched mixed-precision iterative refinement.
//
// MAGMA has iterative refinement only for one matrix at a time
// (magma_dsgesv_gpu, src/zcgesv_gpu.cpp:144-366; magma_dhgesv_iteref_gpu,
// src/dxgesv_gmres_gpu.cpp:1122).  This file applies the same algorithm to a
// whole batch on the device, per matrix:
//   anrm = ||A||_inf, cte = anrm * eps * sqrt(n)           (zcgesv_gpu.cpp:208-209);
//     here anrm is the infinity norm of float(A) with FP32 row sums, which keeps
//     the conversion pass off the FP64 pipe (the tolerance changes by ~n*2^-24)
//   As = float(A) (overflow -> iter = -2), LU of As in FP32 (info > 0 -> iter = -3)
//   X = 0, R = B; repeat: X += float-solve(R); R = B - A X in FP64;
//   converged when, for every right-hand side c, ||R_c||_inf <= ||X_c||_inf * cte
//   (zcgesv_gpu.cpp:266-278), checked first after the initial solve (iter = 0)
//   and after each refinement; ITERMAX = 30 refinements, then iter = -31
//   (zcgesv_gpu.cpp:160-161, 345); failed matrices are re-solved in FP64 with
//   A overwritten by its FP64 factors (zcgesv_gpu.cpp:352-362).
// A second stopping rule is available: the scaled residual
// ||B - A X||_inf / (||A||_inf ||X||_inf n eps) <= tol (the reference tester's
// acceptance metric, testing/testing_zgesv_batched.cpp:131-152).
//
// Everything except the optional FP64 fallback runs without host
// synchronisation; converged matrices drop out of every later launch at the
// cost of one flag read.  The arithmetic is deterministic (fixed fma order in
// the FP64 residual, the oracle's order in the FP32 factor and solves), so the
// CPU oracle reproduces iterates and iteration counts exactly.
#include "common.cuh"
#include "trace.cuh"
#include "convert.cuh"
#include "solve_core.cuh"
#include "chol_core.cuh"

namespace mlu {
template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q);
template <typename T>
magma_int_t chol_factor(int n, T **dA, int lda, int *info, int batch, magma_queue_t q);
template <typename T>
magma_int_t small_gesv(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb, int *info,
                       int batch, magma_queue_t q);
struct VbTune;
template <typename T>
magma_int_t vb_run(const int *m, const int *n, const int *nrhs, int max_m, int max_n, int max_nrhs,
                   T **dA, const int *ldda, int **ipiv, T **dB, const int *lddb, int *info,
                   void *work, int batch, magma_queue_t q, const VbTune *tune_override);
size_t vb_work_bytes(int batch);
template <typename T>
magma_int_t vb_getrs_run(bool trans, const int *n, const int *nrhs, int max_n, int max_nrhs, T **dA,
                         const int *ldda, int **ipiv, T **dB, const int *lddb, int batch,
                         magma_queue_t q);
template <typename T>
magma_int_t ger_neg_vbatched(const int *n, const int *nrhs, int max_n, T **dG, const int *lddg,
                             T **dX, const int *lddx, T **dGA, const int *lddga, int batch,
                             magma_queue_t q);
}  // namespace mlu

extern "C" magma_int_t magma_dgetrf_batched(magma_int_t m, magma_int_t n, double **dA_array,
                                            magma_int_t ldda, magma_int_t **ipiv_array,
                                            magma_int_t *info_array, magma_int_t batchCount,
                                            magma_queue_t queue);
extern "C" magma_int_t magma_dgetrs_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                            double **dA_array, magma_int_t ldda,
                                            magma_int_t **dipiv_array, double **dB_array,
                                            magma_int_t lddb, magma_int_t batchCount,
                                            magma_queue_t queue);
extern "C" magma_int_t magmablas_dger_neg_batched(magma_int_t n, magma_int_t nrhs,
                                                  double **dG_array, magma_int_t lddg,
                                                  double **dX_array, magma_int_t lddx,
                                                  double **dGA_array, magma_int_t lddga,
                                                  magma_int_t batchCount, magma_queue_t queue);

extern "C" magma_int_t magma_sgetrf_batched(magma_int_t m, magma_int_t n, float **dA_array,
                                            magma_int_t ldda, magma_int_t **ipiv_array,
                                            magma_int_t *info_array, magma_int_t batchCount,
                                            magma_queue_t queue);
extern "C" magma_int_t magma_sgetrf_batched_tc(magma_int_t precision, magma_int_t m, magma_int_t n,
                                               float **dA_array, magma_int_t ldda,
                                               magma_int_t **ipiv_array, magma_int_t *info_array,
                                               void *work, size_t *lwork, magma_int_t batchCount,
                                               magma_queue_t queue);
extern "C" magma_int_t magma_sgetrf_batched_tc_status(magma_int_t m, magma_int_t n, void *work,
                                                      magma_int_t batchCount, magma_queue_t queue);
extern "C" magma_int_t magma_dgesv_batched(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                           magma_int_t ldda, magma_int_t **dipiv_array,
                                           double **dB_array, magma_int_t lddb,
                                           magma_int_t *dinfo_array, magma_int_t batchCount,
                                           magma_queue_t queue);

namespace mlu {

constexpr int IR_ROWS = 128;       // rows per CTA in the FP64 kernels
// rows per CTA of the residual: the later refinement passes have only the
// unconverged matrices active, and 64-row CTAs spread them more evenly over
// the SMs (residual class of the refinement benchmark 3.27 -> 3.11 ms per call)
constexpr int IR_RES_ROWS = 64;
constexpr int IR_NRHS_MAX = 16;
constexpr int IR_SOLVE_NR = 8;
constexpr int IR_ACTIVE = 0, IR_CONVERGED = 1, IR_FAILED = 2;
constexpr int IR_FP64 = 3;   // adjoint: the forward solve fell back, A holds FP64 factors

// per-matrix statistics block (8-byte words)
//   [0] anorm bits  [1] state  [2 + par*(2*NRMAX+2) + ...] norms for parity par:
//   rcol[NRMAX], xcol[NRMAX], rrow, xrow
constexpr int IR_STATS_WORDS = 2 + 2 * (2 * IR_NRHS_MAX + 2);

// Sizes of the batch: uniform (the scalars), or per matrix (the arrays, in
// device memory, with the scalars holding the maxima).  Per-matrix scratch
// (FP32 copy, residual, permutation) is laid out for the maxima: matrix k's
// residual column c starts at R + (k * nrhs + c) * n.
struct IrShape {
    int n, nrhs, lda, ldb, ldx;
    const int *n_arr, *nrhs_arr, *lda_arr, *ldb_arr, *ldx_arr;
    __device__ __forceinline__ int N(int k) const { return n_arr ? n_arr[k] : n; }
    __device__ __forceinline__ int NR(int k) const { return nrhs_arr ? nrhs_arr[k] : nrhs; }
    __device__ __forceinline__ int LDA(int k) const { return lda_arr ? lda_arr[k] : lda; }
    __device__ __forceinline__ int LDB(int k) const { return ldb_arr ? ldb_arr[k] : ldb; }
    __device__ __forceinline__ int LDX(int k) const { return ldx_arr ? ldx_arr[k] : ldx; }
};

__device__ __forceinline__ unsigned long long dbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long *norms_of(unsigned long long *st, int par) {
    return st + 2 + par * (2 * IR_NRHS_MAX + 2);
}

// Warp max of a non-negative double, then one atomicMax per warp.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v) {
    unsigned long long b = dbits(v);
    unsigned hi = __reduce_max_sync(FULL, (unsigned)(b >> 32));
    unsigned lo = __reduce_max_sync(FULL, ((unsigned)(b >> 32) == hi) ? (unsigned)b : 0u);
    if ((threadIdx.x & 31) == 0) atomicMax(addr, ((unsigned long long)hi << 32) | lo);
}

// 2^-(e) with e the exponent that puts x * 2^-e in [0.5, 1) (1 for x == 0):
// an exact power-of-two scale factor.
__device__ __forceinline__ double pow2_scale(double x)
{
    if (!(x > 0.0) || isinf(x)) return 1.0;
    const int e = ilogb(x) + 1;
    return ldexp(1.0, -e);
}

// As = float(A), ||A||_inf, R = B, X = 0.  With rowscale != nullptr (FP16
// factorisation) the kernel instead records a power-of-two row scale
// 2^-e_i with max_j |a_ij| 2^-e_i in [0.5, 1) and leaves As to
// ir_colscale_kernel.
__global__ void __launch_bounds__(IR_ROWS)
ir_init_kernel(IrShape sh, double **dA_array, float **dAs_array, int ldas, double **dB_array,
               double **dX_array, double *R, unsigned long long *stats, int *iter,
               double *rowscale)
{
    const int mat = blockIdx.y;
    const int n = sh.N(mat), nrhs = sh.NR(mat);
    const int ldda = sh.LDA(mat), lddb = sh.LDB(mat), lddx = sh.LDX(mat);
    if (n == 0 || nrhs == 0) {                        // nothing to refine
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            stats[(size_t)mat * IR_STATS_WORDS + 1] = IR_CONVERGED;
            iter[mat] = 0;
        }
        return;
    }
    if (blockIdx.x * IR_ROWS >= n) return;            // whole CTA past this matrix
    const int i = blockIdx.x * IR_ROWS + threadIdx.x;
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    const double *A = dA_array[mat];
    float *As = dAs_array[mat];
    double rs = 0.0;
    bool ovf = false;
    if (i < n && rowscale != nullptr) {
        // integer max of |a| (bit patterns order like magnitudes) and FP32 row sums
        unsigned long long mbits = 0ull;
        float rsf = 0.f;
        for (int j = 0; j < n; j++) {
            const double a = A[i + (size_t)j * ldda];
            const unsigned long long ab = (unsigned long long)__double_as_longlong(a) &
                                          0x7fffffffffffffffull;
            mbits = ab > mbits ? ab : mbits;
            rsf += fabsf(d2f_rn_int(a));
        }
        rowscale[(size_t)mat * sh.n + i] = pow2_scale(__longlong_as_double((long long)mbits));
        rs = (double)rsf;
    }
    if (i < n && rowscale == nullptr) {
        // As = float(A) on the integer pipes; ||A||_inf as the FP32 row sums of
        // |float(a_ij)| (j ascending), eight loads in flight per thread
        float rsf = 0.f;
        int j = 0;
        for (; j + 8 <= n; j += 8) {
            double a[8];
#pragma unroll
            for (int u = 0; u < 8; u++) a[u] = A[i + (size_t)(j + u) * ldda];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const float f = d2f_rn_int(a[u]);
                rsf += fabsf(f);
                ovf |= d2f_overflowed(a[u], f);
                As[i + (size_t)(j + u) * ldas] = f;
            }
        }
        for (; j < n; j++) {
            const double a = A[i + (size_t)j * ldda];
            const float f = d2f_rn_int(a);
            rsf += fabsf(f);
            ovf |= d2f_overflowed(a, f);
            As[i + (size_t)j * ldas] = f;
        }
        rs = (double)rsf;
    }
    if (i < n) {
        const double *B = dB_array[mat];
        double *X = dX_array[mat];
        double *Rm = R + (size_t)mat * sh.nrhs * sh.n;
        for (int c = 0; c < nrhs; c++) {
            Rm[i + (size_t)c * sh.n] = B[i + (size_t)c * lddb];
            X[i + (size_t)c * lddx] = 0.0;
        }
    }
    atomic_max_nonneg(&st[0], i < n ? rs : 0.0);
    if (__any_sync(FULL, ovf) && (threadIdx.x & 31) == 0) {
        st[1] = IR_FAILED;
        iter[mat] = -2;
    }
}

// FP16 factorisation: column scale 2^-f_j with max_i |a_ij| 2^-e_i 2^-f_j in
// [0.5, 1), then As = float(a_ij 2^-e_i 2^-f_j).  One thread per column.
__global__ void __launch_bounds__(128)
ir_colscale_kernel(int n, double **dA_array, int ldda, float **dAs_array, int ldas,
                   const double *rowscale, double *colscale)
{
    const int mat = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double *a = dA_array[mat] + (size_t)j * ldda;
    const double *r = rowscale + (size_t)mat * n;
    // scale factors are powers of two, so FP32 arithmetic on float(a) scales exactly
    float cmax = 0.f;
    for (int i = 0; i < n; i++) cmax = fmaxf(cmax, fabsf(d2f_rn_int(a[i])) * (float)r[i]);
    const double c = pow2_scale((double)cmax);
    colscale[(size_t)mat * n + j] = c;
    const float cf = (float)c;
    float *as = dAs_array[mat] + (size_t)j * ldas;
    for (int i = 0; i < n; i++) as[i] = d2f_rn_int(a[i]) * ((float)r[i] * cf);
}

// Convergence test on the norms of parity `par`; called by one thread.
__device__ __forceinline__ bool ir_converged(const unsigned long long *st, int par, int n, int nrhs,
                                             double tol)
{
    const unsigned long long *nm = norms_of(const_cast<unsigned long long *>(st), par);
    const double anrm = bitsd(st[0]);
    const double eps = 1.1102230246251565e-16;   // LAPACK dlamch('Epsilon') = 2^-53
    if (tol > 0.0) {
        // scaled residual ||R||_inf / (||A||_inf ||X||_inf n eps) <= tol
        const double rr = bitsd(nm[2 * IR_NRHS_MAX]), xr = bitsd(nm[2 * IR_NRHS_MAX + 1]);
        return rr <= tol * (anrm * xr * (double)n * eps);
    }
    const double cte = anrm * eps * sqrt((double)n);
    for (int c = 0; c < nrhs; c++) {
        const double rc = bitsd(nm[c]), xc = bitsd(nm[IR_NRHS_MAX + c]);
        if (!(rc <= xc * cte)) return false;
    }
    return true;
}

// check (when it >= 0) + correction solve X += float-solve(R) with the FP32
// factors.  One CTA per (matrix, group of NR right-hand sides).
// Four CTAs per SM (64 registers a thread): the solves are latency-bound, so a
// whole batch of 512 matrices resident at once beats more registers per thread.
// SPD: the factors are the FP32 Cholesky factor L (lower), the correction is
// L L^T d = r (no interchanges, no scaling).
template <int NR, bool TRANS, bool SPD = false, int NT = 256>
__global__ void __launch_bounds__(NT, NT == 256 ? 4 : 2)
ir_solve_kernel(IrShape sh, float **dAs_array, int ldas, const int *perm, double **dX_array,
                const double *R, unsigned long long *stats, int *iter, const int *info, int it,
                double tol, const double *rowscale, const double *colscale)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sB = reinterpret_cast<float *>(smem_raw);
    __shared__ int s_go;
    const int mat = blockIdx.y, tid = threadIdx.x;
    const int n = sh.N(mat), nrhs = sh.NR(mat), lddx = sh.LDX(mat);
    if ((int)blockIdx.x * NR >= nrhs || n == 0) return;   // no right-hand sides for this CTA
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (tid == 0) {
        int go = st[1] == IR_ACTIVE;
        if (go && it < 0 && info != nullptr && info[mat] > 0) {   // FP32 factor hit a zero pivot
            go = 0;
            if (blockIdx.x == 0) { st[1] = IR_FAILED; iter[mat] = -3; }
        }
        if (go && it >= 0 && ir_converged(st, it & 1, n, nrhs, tol)) {
            go = 0;
            if (blockIdx.x == 0) { st[1] = IR_CONVERGED; iter[mat] = it; }
        }
        s_go = go;
    }
    __syncthreads();
    if (!s_go) return;
    // clear the norms the next residual accumulates into
    if (blockIdx.x == 0) {
        unsigned long long *nx = norms_of(st, (it + 1) & 1);
        for (int e = tid; e < 2 * IR_NRHS_MAX + 2; e += blockDim.x) nx[e] = 0ull;
    }
    const int c0 = blockIdx.x * NR;
    const int nr = min(NR, nrhs - c0);
    const double *Rm = R + ((size_t)mat * sh.nrhs + c0) * sh.n;
    const int *pm = SPD ? nullptr : perm + (size_t)mat * sh.n;
    if (SPD) {
        for (int e = tid; e < NR * n; e += blockDim.x) {
            const int c = e / n, i = e % n;
            sB[c * n + i] = __double2float_rn(c < nr ? Rm[i + (size_t)c * sh.n] : 0.0);
        }
    } else if (!TRANS) {
        // row interchanges applied while loading: sB[i] = R[perm[i]]
        for (int e = tid; e < NR * n; e += blockDim.x) {
            const int c = e / n, i = e % n;
            const int p = pm[i];
            const double rv = c < nr ? Rm[p + (size_t)c * sh.n] : 0.0;
            sB[c * n + i] = __double2float_rn(rowscale ? rv * rowscale[(size_t)mat * sh.n + p] : rv);
        }
    } else {
        for (int e = tid; e < NR * n; e += blockDim.x) {
            const int c = e / n, i = e % n;
            sB[c * n + i] = __double2float_rn(c < nr ? Rm[i + (size_t)c * sh.n] : 0.0);
        }
    }
    __syncthreads();
    if (SPD) chol_solve_smem<float, NR>(n, dAs_array[mat], ldas, sB);
    else solve_smem<float, TRANS, NR, true>(n, dAs_array[mat], ldas, nullptr, sB, nr);
    __syncthreads();
    double *X = dX_array[mat] + (size_t)c0 * lddx;
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        const double d = (double)sB[c * n + i];
        // A^T: the interchanges undone on the way out, x[perm[i]] += w[i]
        const int r = (TRANS && !SPD) ? pm[i] : i;
        X[r + (size_t)c * lddx] = X[r + (size_t)c * lddx] +
                                  (colscale ? d * colscale[(size_t)mat * sh.n + i] : d);
    }
}

// Adjoint refinement (A^T GB = G with the forward's FP32 factors): ||A^T||_inf
// as the FP32 column sums of |float(a_ij)| (i ascending), R = G, GB = 0.
// Matrices whose forward solve fell back to FP64 (iter_fwd < 0) are marked
// IR_FP64 and solved afterwards with their FP64 factors.
__global__ void __launch_bounds__(IR_ROWS)
ir_init_adj_kernel(IrShape sh, double **dA_array, double **dG_array, double **dGB_array,
                   double *R, unsigned long long *stats, const int *iter_fwd, int *iter)
{
    const int mat = blockIdx.y;
    const int n = sh.N(mat), nrhs = sh.NR(mat);
    const int ldda = sh.LDA(mat), ldg = sh.LDB(mat), ldgb = sh.LDX(mat);
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (n == 0 || nrhs == 0 || iter_fwd[mat] < 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const bool empty = n == 0 || nrhs == 0;
            st[1] = empty ? IR_CONVERGED : IR_FP64;
            iter[mat] = empty ? 0 : iter_fwd[mat];
        }
        return;
    }
    if (blockIdx.x * IR_ROWS >= n) return;
    const int j = blockIdx.x * IR_ROWS + threadIdx.x;
    float cs = 0.f;
    if (j < n) {
        const double *A = dA_array[mat] + (size_t)j * ldda;
        for (int i = 0; i < n; i++) cs += fabsf(d2f_rn_int(A[i]));
        const double *G = dG_array[mat];
        double *GB = dGB_array[mat];
        double *Rm = R + (size_t)mat * sh.nrhs * sh.n;
        for (int c = 0; c < nrhs; c++) {
            Rm[j + (size_t)c * sh.n] = G[j + (size_t)c * ldg];
            GB[j + (size_t)c * ldgb] = 0.0;
        }
    }
    atomic_max_nonneg(&st[0], j < n ? (double)cs : 0.0);
}

// Gathers the matrices the adjoint refinement did not solve: list 1 all of them
// (GB restarted from G for an FP64 transposed solve), list 2 those whose A
// still needs its FP64 factorisation (the refinement did not converge).
__global__ void ir_compact_adj_kernel(IrShape sh, double **dA_array, int **ipiv_array,
                                      double **dG_array, double **dGB_array,
                                      const unsigned long long *stats, int batch, int *counters,
                                      double **cA, int **cP, double **cGB, int *csize,
                                      double **cA2, int **cP2, int *cidx2, int *csize2)
{
    const int mat = blockIdx.x;
    const unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    const unsigned long long state = st[1];
    if (state != IR_FAILED && state != IR_FP64) return;
    const int n = sh.N(mat), nrhs = sh.NR(mat), ldg = sh.LDB(mat), ldgb = sh.LDX(mat);
    if (threadIdx.x == 0) {
        const int s1 = atomicAdd(&counters[0], 1);
        cA[s1] = dA_array[mat];
        cP[s1] = ipiv_array[mat];
        cGB[s1] = dGB_array[mat];
        if (csize) {
            csize[s1] = n;
            csize[batch + s1] = nrhs;
            csize[2 * batch + s1] = sh.LDA(mat);
            csize[3 * batch + s1] = ldgb;
        }
        if (state == IR_FAILED) {
            const int s2 = atomicAdd(&counters[1], 1);
            cA2[s2] = dA_array[mat];
            cP2[s2] = ipiv_array[mat];
            cidx2[s2] = mat;
            if (csize2) {
                csize2[s2] = n;
                csize2[batch + s2] = sh.LDA(mat);
            }
        }
    }
    const double *G = dG_array[mat];
    double *GB = dGB_array[mat];
    for (int e = threadIdx.x; e < n * nrhs; e += blockDim.x) {
        const int c = e / n, i = e % n;
        GB[i + (size_t)c * ldgb] = G[i + (size_t)c * ldg];
    }
}

// perm[i] = the row of the unpermuted matrix that the sequential interchanges
// ipiv[0..n-1] bring to row i (the interchanges applied to 0..n-1), so a
// solve can gather its right-hand side instead of swapping n times.  One CTA
// per matrix; the interchanges are applied by one thread in shared memory.
__global__ void ir_perm_kernel(IrShape sh, int **ipiv_array, int *perm)
{
    extern __shared__ int s_perm[];
    const int mat = blockIdx.x;
    const int n = sh.N(mat);
    const int *ipiv = ipiv_array[mat];
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_perm[i] = i;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < n; k++) {
            const int p = ipiv[k] - 1;
            if (p != k && MLU_BC2(p, 0, n, 1, 501)) { const int t = s_perm[k]; s_perm[k] = s_perm[p]; s_perm[p] = t; }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[(size_t)mat * sh.n + i] = s_perm[i];
}

// R = B - A X in FP64 (acc = b_i, then acc = fma(-a_ij, x_j, acc) for j = 0..n-1),
// or R = B - A^T X (a_ji in place of a_ij), with the column and row-sum
// infinity norms of R and X.
template <int NR, bool TRANS>
__global__ void __launch_bounds__(IR_RES_ROWS)
ir_residual_kernel(IrShape sh, double **dA_array, double **dB_array, double **dX_array, double *R,
                   unsigned long long *stats, int par)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sX = reinterpret_cast<double *>(smem_raw);   // [n][NR]
    const int mat = blockIdx.y, tid = threadIdx.x;
    const int n = sh.N(mat), nrhs = sh.NR(mat);
    const int ldda = sh.LDA(mat), lddb = sh.LDB(mat), lddx = sh.LDX(mat);
    if (blockIdx.x * IR_RES_ROWS >= n) return;        // whole CTA past this matrix
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (st[1] != IR_ACTIVE) return;
    const double *X = dX_array[mat];
    for (int e = tid; e < n * NR; e += IR_RES_ROWS) {
        const int j = e / NR, c = e % NR;
        sX[e] = c < nrhs ? X[j + (size_t)c * lddx] : 0.0;
    }
    __syncthreads();
    const int i = blockIdx.x * IR_RES_ROWS + tid;
    double acc[NR];
    const double *A = dA_array[mat];
    const double *B = dB_array[mat];
    if (i < n) {
#pragma unroll
        for (int c = 0; c < NR; c++) acc[c] = c < nrhs ? B[i + (size_t)c * lddb] : 0.0;
        // row i of A, or row i of A^T (column i of A, contiguous)
        const double *Ai = TRANS ? A + (size_t)i * ldda : A + i;
        const size_t step = TRANS ? 1 : (size_t)ldda;
        for (int j = 0; j < n; j++) {
            const double a = Ai[(size_t)j * step];
#pragma unroll
            for (int c = 0; c < NR; c++) acc[c] = fma(-a, sX[j * NR + c], acc[c]);
        }
        double *Rm = R + (size_t)mat * sh.nrhs * sh.n;
#pragma unroll
        for (int c = 0; c < NR; c++) if (c < nrhs) Rm[i + (size_t)c * sh.n] = acc[c];
    } else {
#pragma unroll
        for (int c = 0; c < NR; c++) acc[c] = 0.0;
    }
    unsigned long long *nm = norms_of(st, par);
    double rrow = 0.0, xrow = 0.0;
#pragma unroll
    for (int c = 0; c < NR; c++) {
        const double xa = i < n ? fabs(sX[i * NR + c]) : 0.0;
        const double ra = fabs(acc[c]);
        rrow += ra;
        xrow += xa;
        if (c < nrhs) {
            atomic_max_nonneg(&nm[c], ra);
            atomic_max_nonneg(&nm[IR_NRHS_MAX + c], xa);
        }
    }
    atomic_max_nonneg(&nm[2 * IR_NRHS_MAX], rrow);
    atomic_max_nonneg(&nm[2 * IR_NRHS_MAX + 1], xrow);
}

// ---------------------------------------------------------------------------
// GMRES-based refinement (Magma_REFINE_IRGMSTRS of magma_dxgesv_gmres_gpu,
// src/dxgesv_gmres_gpu.cpp:604-780): each refinement iteration solves the
// correction equation A d = r with GMRES right-preconditioned by the
// low-precision LU factors (the reference: FGMRES, src/dgmres_plu_gpu.cpp,
// restart = inner_itermax = 50, relative tolerance innertol = 1e-4, x0 = 0,
// modified Gram-Schmidt, Givens rotations) instead of one solve with them.
// The residual, the update and the stopping rule stay in FP64; the inner
// GMRES runs in FP32 (an FP32 copy of A, FP32 Krylov vectors): FP64 runs at
// 1/64 of the FP32 rate here, and an FP32 inner solver still refines to FP64
// accuracy for condition numbers up to about 1/u_single.  One CTA per matrix
// runs a whole inner solve (at most 8 right-hand sides, one Krylov process
// each), so a refinement iteration is one launch.
constexpr int GM_INNER_MAX = 50;
constexpr float GM_INNER_TOL = 1e-4f;
constexpr int GM_THREADS = 256;
constexpr int GM_WARPS = GM_THREADS / 32;
constexpr int GM_NRHS_MAX = 8;
// A refinement step whose residual 2-norm did not at least halve (any
// right-hand side) ends the refinement of that matrix: it is marked as not
// converged and goes to the FP64 re-solve (the reference instead runs all its
// outer iterations; with FP16/BF16 factors at kappa ~1e6 the GMRES correction
// stalls and every further iteration is wasted).
constexpr double GM_STALL = 0.5;

// A32 = float(A) (uniform batch, rows coalesced)
__global__ void __launch_bounds__(IR_ROWS)
gm_a32_kernel(IrShape sh, double **dA_array, float *A32, int ldas)
{
    const int mat = blockIdx.y;
    const int i = blockIdx.x * IR_ROWS + threadIdx.x;
    if (i >= sh.n) return;
    const double *A = dA_array[mat];
    float *D = A32 + (size_t)mat * sh.n * ldas;
    for (int j = 0; j < sh.n; j++) D[i + (size_t)j * ldas] = __double2float_rn(A[i + (size_t)j * sh.lda]);
}

// Block sums of NR per-thread partials, lane order then warp order (the same
// order on every call); the sums land in out[] for every thread.
template <typename F, int NR>
__device__ __forceinline__ void gm_block_sum(F (&v)[NR], F (*red)[NR], F *out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NR; c++) {
        F x = v[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
        v[c] = x;
    }
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < NR; c++) red[warp][c] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < NR) {
        F t = F(0);
        for (int w = 0; w < GM_WARPS; w++) t += red[w][threadIdx.x];
        out[threadIdx.x] = t;
    }
    __syncthreads();
}

template <int NR>
__host__ __device__ inline size_t gm_smem_bytes(int n)
{
    const int m = n < GM_INNER_MAX ? n : GM_INNER_MAX;
    return sizeof(float) * ((size_t)2 * NR * n + (size_t)NR * (m + 1) * m + (size_t)NR * (3 * m + 1));
}

// check (as ir_solve_kernel) + GMRES correction X += d for the nrhs <= NR
// right-hand sides of one matrix.  V: per right-hand side GM_INNER_MAX+1 FP32
// vectors of n.
template <int NR>
__global__ void __launch_bounds__(GM_THREADS)
gm_correction_kernel(IrShape sh, float **dAs_array, int ldas, const int *perm, const float *A32,
                     double **dX_array, const double *R, unsigned long long *stats, int *iter,
                     int *inner_total, int it, double tol, const double *rowscale,
                     const double *colscale, float *Vbase, double *beta_prev, int itermax)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float s_red[GM_WARPS][NR], s_sum[NR];
    __shared__ double s_red64[GM_WARPS][NR], s_sum64[NR];
    __shared__ int s_go, s_act[NR], s_k[NR], s_any;
    const int mat = blockIdx.y, tid = threadIdx.x;
    const int n = sh.N(mat), nrhs = sh.NR(mat), lddx = sh.LDX(mat);
    if (n == 0 || nrhs == 0) return;
    const int m = min(GM_INNER_MAX, n);
    float *sB = reinterpret_cast<float *>(smem_raw);   // [NR][n]: preconditioner input / output
    float *sW = sB + NR * n;                           // [NR][n]: Arnoldi vector
    float *sH = sW + NR * n;                           // [NR][m+1][m]: Hessenberg matrices
    float *sCs = sH + NR * (m + 1) * m;                // [NR][m]
    float *sSn = sCs + NR * m;                         // [NR][m]
    float *sRs = sSn + NR * m;                         // [NR][m+1]: rotated right-hand side, then y
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (tid == 0) {
        int go = st[1] == IR_ACTIVE;
        if (go && ir_converged(st, it & 1, n, nrhs, tol)) {
            go = 0;
            st[1] = IR_CONVERGED;
            iter[mat] = inner_total[mat];
        }
        s_go = go;
    }
    __syncthreads();
    if (!s_go) return;
    {
        unsigned long long *nx = norms_of(st, (it + 1) & 1);
        for (int e = tid; e < 2 * IR_NRHS_MAX + 2; e += GM_THREADS) nx[e] = 0ull;
    }
    const int nr = min(NR, nrhs);
    const double *Rm = R + (size_t)mat * sh.nrhs * sh.n;
    float *Vm = Vbase + (size_t)mat * sh.nrhs * (GM_INNER_MAX + 1) * sh.n;
    const int *pm = perm + (size_t)mat * sh.n;
    const float *Am = A32 + (size_t)mat * sh.n * ldas;
    const float *LU = dAs_array[mat];
    const double *rsc = rowscale ? rowscale + (size_t)mat * sh.n : nullptr;
    const double *csc = colscale ? colscale + (size_t)mat * sh.n : nullptr;
    auto V = [&](int c, int j) { return Vm + ((size_t)c * (GM_INNER_MAX + 1) + j) * sh.n; };

    // beta_c = ||r_c||_2 in FP64; v_0 = r_c / beta_c; the inner system is
    // A z = v_0 with ||v_0|| = 1 (rs_0 = 1), and d = beta_c z
    {
        double part[NR];
#pragma unroll
        for (int c = 0; c < NR; c++) part[c] = 0.0;
        for (int r = tid; r < n; r += GM_THREADS)
#pragma unroll
            for (int c = 0; c < NR; c++)
                if (c < nr) { const double x = Rm[r + (size_t)c * sh.n]; part[c] = fma(x, x, part[c]); }
        gm_block_sum<double, NR>(part, s_red64, s_sum64);
    }
    double beta[NR];
#pragma unroll
    for (int c = 0; c < NR; c++) beta[c] = sqrt(s_sum64[c]);
    if (tid == 0) {
        double *bp = beta_prev + (size_t)mat * NR;
        int stall = 0;
        for (int c = 0; c < nr; c++) {
            if (it > 0 && !(beta[c] <= GM_STALL * bp[c])) stall = 1;
            bp[c] = beta[c];
        }
        if (stall) {
            st[1] = IR_FAILED;
            iter[mat] = -itermax - 1;
        }
        s_go = !stall;
    }
    __syncthreads();
    if (!s_go) return;
    for (int r = tid; r < n; r += GM_THREADS)
#pragma unroll
        for (int c = 0; c < NR; c++)
            if (c < nr) V(c, 0)[r] = beta[c] > 0.0 ? __double2float_rn(Rm[r + (size_t)c * sh.n] / beta[c]) : 0.f;
    if (tid < NR) {
        s_act[tid] = tid < nr && beta[tid] > 0.0 && isfinite(beta[tid]);
        s_k[tid] = 0;
        sRs[tid * (m + 1)] = 1.f;
    }
    __syncthreads();
    for (int i = 0; i < m; i++) {
        if (tid == 0) {
            int a = 0;
#pragma unroll
            for (int c = 0; c < NR; c++) a |= s_act[c];
            s_any = a;
        }
        __syncthreads();
        if (!s_any) break;
        // z = M^{-1} v_i: row interchanges (and the FP16 form's row scale) on
        // the way in, the column scale on the way out
        for (int e = tid; e < NR * n; e += GM_THREADS) {
            const int c = e / n, q = e % n, p = pm[q];
            float x = 0.f;
            if (c < nr) {
                x = V(c, i)[p];
                if (rsc) x *= (float)rsc[p];
            }
            sB[c * n + q] = x;
        }
        __syncthreads();
        solve_smem<float, false, NR>(n, LU, ldas, nullptr, sB, nr);
        __syncthreads();
        if (csc) {
            for (int e = tid; e < NR * n; e += GM_THREADS) sB[e] *= (float)csc[e % n];
            __syncthreads();
        }
        // w = A z
        for (int r = tid; r < n; r += GM_THREADS) {
            float acc[NR];
#pragma unroll
            for (int c = 0; c < NR; c++) acc[c] = 0.f;
            const float *Ar = Am + r;
#pragma unroll 8
            for (int j = 0; j < n; j++) {
                const float a = Ar[(size_t)j * ldas];
#pragma unroll
                for (int c = 0; c < NR; c++) acc[c] = fmaf(a, sB[c * n + j], acc[c]);
            }
#pragma unroll
            for (int c = 0; c < NR; c++) sW[c * n + r] = acc[c];
        }
        // modified Gram-Schmidt against v_0..v_i
        for (int j = 0; j <= i; j++) {
            float part[NR];
#pragma unroll
            for (int c = 0; c < NR; c++) part[c] = 0.f;
            for (int r = tid; r < n; r += GM_THREADS)
#pragma unroll
                for (int c = 0; c < NR; c++)
                    if (c < nr) part[c] = fmaf(sW[c * n + r], V(c, j)[r], part[c]);
            gm_block_sum<float, NR>(part, s_red, s_sum);
            for (int r = tid; r < n; r += GM_THREADS)
#pragma unroll
                for (int c = 0; c < NR; c++)
                    if (c < nr) sW[c * n + r] = fmaf(-s_sum[c], V(c, j)[r], sW[c * n + r]);
            if (tid < NR) sH[((size_t)tid * (m + 1) + j) * m + i] = s_sum[tid];
        }
        {
            float part[NR];
#pragma unroll
            for (int c = 0; c < NR; c++) part[c] = 0.f;
            for (int r = tid; r < n; r += GM_THREADS)
#pragma unroll
                for (int c = 0; c < NR; c++)
                    if (c < nr) part[c] = fmaf(sW[c * n + r], sW[c * n + r], part[c]);
            gm_block_sum<float, NR>(part, s_red, s_sum);
        }
        float hn[NR];
#pragma unroll
        for (int c = 0; c < NR; c++) hn[c] = sqrtf(s_sum[c]);
        if (i + 1 <= m)
            for (int r = tid; r < n; r += GM_THREADS)
#pragma unroll
                for (int c = 0; c < NR; c++)
                    if (c < nr) V(c, i + 1)[r] = hn[c] > 0.f ? sW[c * n + r] / hn[c] : 0.f;
        if (tid < NR) sH[((size_t)tid * (m + 1) + i + 1) * m + i] = hn[tid];
        __syncthreads();
        // Givens rotations, one thread per right-hand side
        if (tid < nr && s_act[tid]) {
            const int c = tid;
            float *H = sH + (size_t)c * (m + 1) * m;
            float *cs = sCs + c * m, *sn = sSn + c * m, *rs = sRs + c * (m + 1);
            for (int j = 0; j < i; j++) {
                const float t = H[j * m + i], u = H[(j + 1) * m + i];
                H[j * m + i] = cs[j] * t + sn[j] * u;
                H[(j + 1) * m + i] = -sn[j] * t + cs[j] * u;
            }
            const float a = H[i * m + i], b = H[(i + 1) * m + i];
            float gam = hypotf(a, b);
            if (gam == 0.f) gam = 1e-30f;
            cs[i] = a / gam;
            sn[i] = b / gam;
            rs[i + 1] = -sn[i] * rs[i];
            rs[i] = cs[i] * rs[i];
            H[i * m + i] = cs[i] * a + sn[i] * b;
            s_k[c] = i + 1;
            if (!(fabsf(rs[i + 1]) > GM_INNER_TOL) || b == 0.f) s_act[c] = 0;
        }
        __syncthreads();
    }
    // y = H^{-1} rs (upper triangular, k x k)
    if (tid < nr && s_k[tid] > 0) {
        const int c = tid, k = s_k[c];
        const float *H = sH + (size_t)c * (m + 1) * m;
        float *rs = sRs + c * (m + 1);
        for (int kk = k - 1; kk >= 0; kk--) {
            float t = rs[kk];
            for (int j = kk + 1; j < k; j++) t = fmaf(-H[kk * m + j], rs[j], t);
            rs[kk] = t / H[kk * m + kk];
        }
    }
    __syncthreads();
    // d = beta M^{-1} (V y)
    for (int e = tid; e < NR * n; e += GM_THREADS) {
        const int c = e / n, q = e % n, p = pm[q];
        float t = 0.f;
        if (c < nr) {
            for (int j = 0; j < s_k[c]; j++) t = fmaf(sRs[c * (m + 1) + j], V(c, j)[p], t);
            if (rsc) t *= (float)rsc[p];
        }
        sB[c * n + q] = t;
    }
    __syncthreads();
    solve_smem<float, false, NR>(n, LU, ldas, nullptr, sB, nr);
    __syncthreads();
    double *X = dX_array[mat];
    for (int e = tid; e < nr * n; e += GM_THREADS) {
        const int c = e / n, q = e % n;
        if (s_k[c] == 0) continue;
        const double d = (double)sB[c * n + q];
        X[q + (size_t)c * lddx] += beta[c] * (csc ? d * csc[q] : d);
    }
    if (tid == 0) {
        int kmax = 0;
#pragma unroll
        for (int c = 0; c < NR; c++) kmax = max(kmax, s_k[c]);
        inner_total[mat] += kmax;
    }
}

__global__ void ir_final_kernel(IrShape sh, unsigned long long *stats, int *iter, int itermax,
                                double tol, int batch, int *failed_count,
                                const int *inner_total = nullptr)
{
    const int mat = blockIdx.x * blockDim.x + threadIdx.x;
    if (mat >= batch) return;
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (st[1] == IR_ACTIVE) {
        if (ir_converged(st, itermax & 1, sh.N(mat), sh.NR(mat), tol)) {
            st[1] = IR_CONVERGED;
            iter[mat] = inner_total ? inner_total[mat] : itermax;
        } else {
            st[1] = IR_FAILED;
            iter[mat] = -itermax - 1;
        }
    }
    if (st[1] == IR_FAILED || st[1] == IR_FP64) atomicAdd(failed_count, 1);
}

// Gathers the failed matrices into compact pointer arrays and restarts their
// X from B for the FP64 re-solve.
__global__ void ir_compact_kernel(IrShape sh, double **dA_array, int **ipiv_array,
                                  double **dB_array, double **dX_array,
                                  const unsigned long long *stats, int batch, int *counter,
                                  double **cA, int **cP, double **cX, int *cidx, int *csize)
{
    const int mat = blockIdx.x;
    const unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (st[1] != IR_FAILED) return;
    const int n = sh.N(mat), nrhs = sh.NR(mat), lddb = sh.LDB(mat), lddx = sh.LDX(mat);
    __shared__ int slot;
    if (threadIdx.x == 0) {
        slot = atomicAdd(counter, 1);
        cA[slot] = dA_array[mat];
        cP[slot] = ipiv_array ? ipiv_array[mat] : nullptr;   // no pivots: the SPD form
        cX[slot] = dX_array[mat];
        cidx[slot] = mat;
        if (csize) {          // variable sizes: n, nrhs, ldda, lddx of the compacted batch
            csize[slot] = n;
            csize[batch + slot] = nrhs;
            csize[2 * batch + slot] = sh.LDA(mat);
            csize[3 * batch + slot] = lddx;
        }
    }
    const double *B = dB_array[mat];
    double *X = dX_array[mat];
    for (int e = threadIdx.x; e < n * nrhs; e += blockDim.x) {
        const int c = e / n, i = e % n;
        X[i + (size_t)c * lddx] = B[i + (size_t)c * lddb];
    }
}

__global__ void ir_scatter_info_kernel(int count, const int *cidx, const int *cinfo, int *info)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) info[cidx[k]] = cinfo[k];
}

__global__ void set_float_pointers(float **out, float *base, size_t stride, int batch, int *ld_arr,
                                   int ld)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < batch) {
        out[k] = base + (size_t)k * stride;
        if (ld_arr) ld_arr[k] = ld;
    }
}

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct IrLayout {
    size_t stats, count, asp, as, r, perm, ca, cp, cx, cidx, cinfo, rsc, csc, tc, tc_bytes;
    size_t ldas_arr, csize, vbw, ca2, cp2, csize2, gm_a32, gm_v, gm_inner, gm_beta, total;
    int ldas;
};

// Workspace of a refinement over `batch` matrices of order <= n with <= nrhs
// right-hand sides; `vb` adds the arrays of a variable-size batch.
static IrLayout ir_layout(int n, int nrhs, int batch, int prec = 900, bool vb = false,
                          int solver = 920)
{
    IrLayout L;
    L.ldas = (n + 31) & ~31;
    size_t o = 0;
    L.stats = o; o = align256(o + (size_t)batch * IR_STATS_WORDS * 8);
    L.count = o; o = align256(o + 16);
    L.asp = o;   o = align256(o + (size_t)batch * sizeof(float *));
    L.as = o;    o = align256(o + (size_t)batch * n * L.ldas * sizeof(float));
    L.r = o;     o = align256(o + (size_t)batch * nrhs * n * sizeof(double));
    L.perm = o;  o = align256(o + (size_t)batch * n * sizeof(int));
    L.ca = o;    o = align256(o + (size_t)batch * sizeof(double *));
    L.cp = o;    o = align256(o + (size_t)batch * sizeof(int *));
    L.cx = o;    o = align256(o + (size_t)batch * sizeof(double *));
    L.cidx = o;  o = align256(o + (size_t)batch * sizeof(int));
    L.cinfo = o; o = align256(o + (size_t)batch * sizeof(int));
    L.ca2 = o;   o = align256(o + (size_t)batch * sizeof(double *));   // adjoint fallback lists
    L.cp2 = o;   o = align256(o + (size_t)batch * sizeof(int *));
    L.ldas_arr = L.csize = L.csize2 = L.vbw = o;
    if (vb) {
        L.csize2 = o;   o = align256(o + 2 * (size_t)batch * sizeof(int));
        L.ldas_arr = o; o = align256(o + (size_t)batch * sizeof(int));
        L.csize = o;    o = align256(o + 4 * (size_t)batch * sizeof(int));
        L.vbw = o;      o = align256(o + vb_work_bytes(batch));
    }
    L.rsc = L.csc = L.tc = o;
    L.tc_bytes = 0;
    if (prec == 905) {
        L.rsc = o; o = align256(o + (size_t)batch * n * sizeof(double));
        L.csc = o; o = align256(o + (size_t)batch * n * sizeof(double));
    }
    if (prec != 900) {
        size_t tcb = 0;
        magma_sgetrf_batched_tc(prec, n, n, nullptr, mlu_max(1, (n + 31) & ~31), nullptr, nullptr,
                                nullptr, &tcb, batch, nullptr);
        o = (o + 1023) & ~(size_t)1023;
        L.tc = o;
        L.tc_bytes = tcb;
        o = align256(o + tcb);
    }
    L.gm_a32 = L.gm_v = L.gm_inner = L.gm_beta = o;
    if (solver == 922) {   // GMRES refinement: FP32 copy of A, Krylov vectors, inner counts
        L.gm_a32 = o;   o = align256(o + (size_t)batch * n * L.ldas * sizeof(float));
        L.gm_v = o;     o = align256(o + (size_t)batch * nrhs * (GM_INNER_MAX + 1) * n * sizeof(float));
        L.gm_inner = o; o = align256(o + (size_t)batch * sizeof(int));
        L.gm_beta = o;  o = align256(o + (size_t)batch * GM_NRHS_MAX * sizeof(double));
    }
    L.total = o;
    return L;
}

template <int NR, bool TRANS>
static void launch_residual(const IrShape &sh, double **dA, double **dB, double **dX, double *R,
                            unsigned long long *stats, int par, int batch, cudaStream_t s)
{
    const size_t smem = (size_t)sh.n * NR * sizeof(double);
    static size_t dyn_cache[MLU_MAX_DEVICES];
    mlu_device_cached(dyn_cache, [] { return mlu_allow_dynamic_smem(ir_residual_kernel<NR, TRANS>); });
    MLU_LAUNCH(mlu::KC_IR_RESIDUAL, s,
               ir_residual_kernel<NR, TRANS><<<dim3((sh.n + IR_RES_ROWS - 1) / IR_RES_ROWS, batch), IR_RES_ROWS,
                                               smem, s>>>(sh, dA, dB, dX, R, stats, par));
}

template <bool TRANS>
static void residual(const IrShape &sh, double **dA, double **dB, double **dX, double *R,
                     unsigned long long *stats, int par, int batch, cudaStream_t s)
{
    if (sh.nrhs <= 1)      launch_residual<1, TRANS>(sh, dA, dB, dX, R, stats, par, batch, s);
    else if (sh.nrhs <= 2) launch_residual<2, TRANS>(sh, dA, dB, dX, R, stats, par, batch, s);
    else if (sh.nrhs <= 4) launch_residual<4, TRANS>(sh, dA, dB, dX, R, stats, par, batch, s);
    else if (sh.nrhs <= 8) launch_residual<8, TRANS>(sh, dA, dB, dX, R, stats, par, batch, s);
    else                   launch_residual<16, TRANS>(sh, dA, dB, dX, R, stats, par, batch, s);
}

// SMs of the current device (cached per device).
static int ir_sm_count()
{
    static size_t cache[MLU_MAX_DEVICES];
    return (int)mlu_device_cached(cache, [] {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return (size_t)sms;
    });
}

// check + correction solve of refinement iteration `it` (-1: the initial solve)
template <bool TRANS>
static void correction_solve(const IrShape &sh, float **As_array, int ldas, const int *perm,
                             double **dX, const double *R, unsigned long long *stats, int *iter,
                             const int *info, int it, double tol, const double *rsc,
                             const double *csc, int batch, cudaStream_t s, bool spd = false)
{
    const int snr = sh.nrhs <= 4 ? 4 : IR_SOLVE_NR;   // right-hand sides per CTA
    const size_t ssmem = (size_t)snr * sh.n * sizeof(float);
    const dim3 grid(mlu_ceildiv(sh.nrhs, snr), batch);
    if (spd) {
        if (snr == 4)
            MLU_LAUNCH(mlu::KC_IR_SOLVE, s, ir_solve_kernel<4, false, true><<<grid, 256, ssmem, s>>>(
                sh, As_array, ldas, perm, dX, R, stats, iter, info, it, tol, nullptr, nullptr));
        else
            MLU_LAUNCH(mlu::KC_IR_SOLVE, s, ir_solve_kernel<IR_SOLVE_NR, false, true><<<grid, 256, ssmem, s>>>(
                sh, As_array, ldas, perm, dX, R, stats, iter, info, it, tol, nullptr, nullptr));
        return;
    }
    // a batch that two CTAs per SM hold at once gets 512-thread CTAs: each matrix's
    // updates below its diagonal blocks spread over twice the threads (the largest
    // matrix's chain of blocks is the launch's critical path)
    if ((size_t)grid.x * grid.y <= 2 * (size_t)ir_sm_count()) {
        if (snr == 4)
            MLU_LAUNCH(mlu::KC_IR_SOLVE, s, ir_solve_kernel<4, TRANS, false, 512><<<grid, 512, ssmem, s>>>(
                sh, As_array, ldas, perm, dX, R, stats, iter, info, it, tol, rsc, csc));
        else
            MLU_LAUNCH(mlu::KC_IR_SOLVE, s, ir_solve_kernel<IR_SOLVE_NR, TRANS, false, 512><<<grid, 512, ssmem, s>>>(
                sh, As_array, ldas, perm, dX, R, stats, iter, info, it, tol, rsc, csc));
        return;
    }
    if (snr == 4)
        MLU_LAUNCH(mlu::KC_IR_SOLVE, s, ir_solve_kernel<4, TRANS><<<grid, 256, ssmem, s>>>(
            sh, As_array, ldas, perm, dX, R, stats, iter, info, it, tol, rsc, csc));
    else
        MLU_LAUNCH(mlu::KC_IR_SOLVE, s, ir_solve_kernel<IR_SOLVE_NR, TRANS><<<grid, 256, ssmem, s>>>(
            sh, As_array, ldas, perm, dX, R, stats, iter, info, it, tol, rsc, csc));
}

// Right-hand sides per CTA of the residual kernel for nrhs (residual()) and of
// the correction solve (correction_solve()).
static int residual_nr(int nrhs) { return nrhs <= 1 ? 1 : nrhs <= 2 ? 2 : nrhs <= 4 ? 4 : nrhs <= 8 ? 8 : 16; }
static int solve_nr(int nrhs) { return nrhs <= 4 ? 4 : IR_SOLVE_NR; }
constexpr size_t IR_RESIDUAL_SMEM_MAX = 200 * 1024;   // X rows of the residual, in shared memory

static size_t solve_dyn_max();

// The refinement keeps one matrix's right-hand sides in shared memory: n *
// residual_nr(nrhs) doubles for the residual and n * solve_nr(nrhs) floats for
// the correction solve.  False (with a message naming the largest order for
// this nrhs) when n is too large for that.
static bool ir_fits(const char *name, int n, int nrhs)
{
    const size_t rb = (size_t)residual_nr(nrhs) * sizeof(double), sb = (size_t)solve_nr(nrhs) * sizeof(float);
    const size_t smax = solve_dyn_max();
    if ((size_t)n * rb <= IR_RESIDUAL_SMEM_MAX && (size_t)n * sb <= smax) return true;
    const size_t nmax = min(IR_RESIDUAL_SMEM_MAX / rb, smax / sb);
    fprintf(stderr, "%s: order n=%d with nrhs=%d does not fit the refinement's shared-memory right-hand "
                    "sides; the largest order for this nrhs is %zu\n", name, n, nrhs, nmax);
    return false;
}

static size_t gm_dyn_max()
{
    static size_t cache[MLU_MAX_DEVICES];
    return mlu_device_cached(cache, [] {
        return min(mlu_allow_dynamic_smem(gm_correction_kernel<4>),
                   mlu_allow_dynamic_smem(gm_correction_kernel<8>));
    });
}

static size_t solve_dyn_max()
{
    static size_t cache[MLU_MAX_DEVICES];
    return mlu_device_cached(cache, [] {
        return min(min(min(mlu_allow_dynamic_smem(ir_solve_kernel<IR_SOLVE_NR, false>),
                           mlu_allow_dynamic_smem(ir_solve_kernel<4, false>)),
                       min(mlu_allow_dynamic_smem(ir_solve_kernel<IR_SOLVE_NR, true>),
                           mlu_allow_dynamic_smem(ir_solve_kernel<4, true>))),
                   min(min(mlu_allow_dynamic_smem(ir_solve_kernel<IR_SOLVE_NR, false, true>),
                           mlu_allow_dynamic_smem(ir_solve_kernel<4, false, true>)),
                       min(min(mlu_allow_dynamic_smem(ir_solve_kernel<IR_SOLVE_NR, false, false, 512>),
                               mlu_allow_dynamic_smem(ir_solve_kernel<4, false, false, 512>)),
                           min(mlu_allow_dynamic_smem(ir_solve_kernel<IR_SOLVE_NR, true, false, 512>),
                               mlu_allow_dynamic_smem(ir_solve_kernel<4, true, false, 512>)))));
    });
}

}  // namespace mlu

using namespace mlu;

// The refinement driver for factorisation precision `prec`: 900 FP32
// (Magma_PREC_SS), 905 FP16 tensor-core updates (Magma_PREC_SHT, with
// power-of-two row and column scaling), 930 BF16 tensor-core updates.  `sh`
// holds uniform sizes, or per-matrix size arrays with their maxima (FP32
// factorisation by the persistent variable-size kernel).  Argument checks are
// the caller's.
static magma_int_t
ir_run(int prec, const IrShape &sh, double **dA_array, magma_int_t **dipiv_array,
       double **dB_array, double **dX_array, magma_int_t *dinfo_array, magma_int_t *diter_array,
       magma_int_t itermax, double tol, magma_int_t fallback, void *work, size_t *lwork,
       magma_int_t batchCount, magma_queue_t queue, int solver = 920, bool spd = false)
{
    const bool vb = sh.n_arr != nullptr;
    const int n = sh.n, nrhs = sh.nrhs;
    const bool gm = solver == 922;
    if (spd && (vb || gm || prec != 900)) return MAGMA_ERR_NOT_SUPPORTED;
    const IrLayout L = ir_layout(n, nrhs, mlu_max(batchCount, 0), prec, vb, solver);
    if (work == nullptr) {          // workspace query
        *lwork = L.total;
        return 0;
    }
    if (*lwork < L.total) return -15;
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    // shared-memory limits of the correction solve and the residual kernels
    if (!ir_fits("magma_dxgesv_batched", n, nrhs)) return MAGMA_ERR_NOT_SUPPORTED;
    if (gm && (vb || nrhs > GM_NRHS_MAX || gm_smem_bytes<GM_NRHS_MAX>(n) > gm_dyn_max()))
        return MAGMA_ERR_NOT_SUPPORTED;

    cudaStream_t s = queue->stream;
    char *w = (char *)work;
    unsigned long long *stats = (unsigned long long *)(w + L.stats);
    int *count = (int *)(w + L.count);
    float **As_array = (float **)(w + L.asp);
    float *As = (float *)(w + L.as);
    double *R = (double *)(w + L.r);
    int *ldas_arr = vb ? (int *)(w + L.ldas_arr) : nullptr;

    cudaMemsetAsync(w, 0, L.asp, s);   // stats, counters
    MLU_LAUNCH(mlu::KC_OTHER, s, set_float_pointers<<<mlu_ceildiv(batchCount, 256), 256, 0, s>>>(
        As_array, As, (size_t)n * L.ldas, batchCount, ldas_arr, L.ldas));
    double *rsc = prec == 905 ? (double *)(w + L.rsc) : nullptr;
    double *csc = prec == 905 ? (double *)(w + L.csc) : nullptr;
    const dim3 rows_grid((n + IR_ROWS - 1) / IR_ROWS, batchCount);
    MLU_LAUNCH(mlu::KC_IR_INIT, s, ir_init_kernel<<<rows_grid, IR_ROWS, 0, s>>>(
        sh, dA_array, As_array, L.ldas, dB_array, dX_array, R, stats, diter_array, rsc));
    if (rsc)
        MLU_LAUNCH(mlu::KC_IR_INIT, s, ir_colscale_kernel<<<dim3((n + 127) / 128, batchCount), 128, 0, s>>>(
            n, dA_array, sh.lda, As_array, L.ldas, rsc, csc));
    magma_int_t rc;
    if (spd) {
        rc = chol_factor<float>(n, As_array, L.ldas, dinfo_array, batchCount, queue);
    } else if (vb) {
        rc = vb_run<float>(sh.n_arr, sh.n_arr, nullptr, n, n, 0, As_array, ldas_arr, dipiv_array,
                           nullptr, nullptr, dinfo_array, w + L.vbw, batchCount, queue, nullptr);
    } else if (prec == 900) {
        rc = magma_sgetrf_batched(n, n, As_array, L.ldas, dipiv_array, dinfo_array, batchCount,
                                  queue);
    } else {
        size_t tcb = L.tc_bytes;
        rc = magma_sgetrf_batched_tc(prec, n, n, As_array, L.ldas, dipiv_array, dinfo_array,
                                     w + L.tc, &tcb, batchCount, queue);
    }
    if (rc != 0) return rc;
    int *perm = (int *)(w + L.perm);
    if (!spd)
        MLU_LAUNCH(mlu::KC_OTHER, s, ir_perm_kernel<<<batchCount, 256, (size_t)n * sizeof(int), s>>>(
            sh, dipiv_array, perm));
    auto solve = [&](int it) {
        correction_solve<false>(sh, As_array, L.ldas, perm, dX_array, R, stats, diter_array,
                                dinfo_array, it, tol, rsc, csc, batchCount, s, spd);
    };
    float *A32 = gm ? (float *)(w + L.gm_a32) : nullptr;
    float *Vk = gm ? (float *)(w + L.gm_v) : nullptr;
    int *inner = gm ? (int *)(w + L.gm_inner) : nullptr;
    double *beta_prev = gm ? (double *)(w + L.gm_beta) : nullptr;
    if (gm) {
        cudaMemsetAsync(inner, 0, (size_t)batchCount * sizeof(int), s);
        MLU_LAUNCH(mlu::KC_IR_INIT, s, gm_a32_kernel<<<rows_grid, IR_ROWS, 0, s>>>(
            sh, dA_array, A32, L.ldas));
    }
    auto gmres = [&](int it) {
        if (nrhs <= 4)
            MLU_LAUNCH(mlu::KC_IR_SOLVE, s, gm_correction_kernel<4><<<dim3(1, batchCount), GM_THREADS,
                                                                      gm_smem_bytes<4>(n), s>>>(
                sh, As_array, L.ldas, perm, A32, dX_array, R, stats, diter_array, inner, it, tol,
                rsc, csc, Vk, beta_prev, itermax));
        else
            MLU_LAUNCH(mlu::KC_IR_SOLVE, s, gm_correction_kernel<8><<<dim3(1, batchCount), GM_THREADS,
                                                                      gm_smem_bytes<8>(n), s>>>(
                sh, As_array, L.ldas, perm, A32, dX_array, R, stats, diter_array, inner, it, tol,
                rsc, csc, Vk, beta_prev, itermax));
    };
    solve(-1);
    residual<false>(sh, dA_array, dB_array, dX_array, R, stats, 0, batchCount, s);
    for (int it = 0; it < itermax; it++) {
        if (gm) gmres(it);
        else solve(it);
        residual<false>(sh, dA_array, dB_array, dX_array, R, stats, (it + 1) & 1, batchCount, s);
    }
    MLU_LAUNCH(mlu::KC_OTHER, s, ir_final_kernel<<<mlu_ceildiv(batchCount, 256), 256, 0, s>>>(
        sh, stats, diter_array, itermax, tol, batchCount, count, inner));
    MLU_CHECK_LAUNCH();
    if (!fallback) return 0;

    int failed = 0;
    cudaMemcpyAsync(&failed, count, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    if (prec != 900 && magma_sgetrf_batched_tc_status(n, n, w + L.tc, batchCount, queue) != 0)
        return MAGMA_ERR_UNKNOWN;   // a tensor-pipeline wait timed out
    if (failed == 0) return 0;
    double **cA = (double **)(w + L.ca);
    int **cP = (int **)(w + L.cp);
    double **cX = (double **)(w + L.cx);
    int *cidx = (int *)(w + L.cidx);
    int *cinfo = (int *)(w + L.cinfo);
    int *csize = vb ? (int *)(w + L.csize) : nullptr;
    cudaMemsetAsync(count + 1, 0, sizeof(int), s);
    MLU_LAUNCH(mlu::KC_OTHER, s, ir_compact_kernel<<<batchCount, 256, 0, s>>>(
        sh, dA_array, dipiv_array, dB_array, dX_array, stats, batchCount, count + 1, cA, cP, cX,
        cidx, csize));
    if (spd)
        rc = magma_dposv_batched(MagmaLower, n, nrhs, cA, sh.lda, cX, sh.ldx, cinfo, failed, queue);
    else if (vb)
        rc = vb_run<double>(csize, csize, csize + batchCount, n, n, nrhs, cA, csize + 2 * batchCount,
                            cP, cX, csize + 3 * batchCount, cinfo, w + L.vbw, failed, queue,
                            nullptr);
    else
        rc = magma_dgesv_batched(n, nrhs, cA, sh.lda, cP, cX, sh.ldx, cinfo, failed, queue);
    if (rc != 0) return rc;
    MLU_LAUNCH(mlu::KC_OTHER, s, ir_scatter_info_kernel<<<mlu_ceildiv(failed, 256), 256, 0, s>>>(
        failed, cidx, cinfo, dinfo_array));
    MLU_CHECK_LAUNCH();
    return 0;
}

// The FP64 part of the adjoint: compacts the matrices the refinement left
// unsolved (list 1: all, GB restarted from G; list 2: those still needing an
// FP64 factorisation), factors list 2 in place and solves list 1 with A^T.
static magma_int_t adjoint_fp64_solves(const IrShape &sh, const IrLayout &L, char *w,
                                       double **dA_array, magma_int_t **dipiv_array,
                                       double **dG_array, double **dGB_array,
                                       magma_int_t *dinfo_array, int batchCount,
                                       magma_queue_t queue)
{
    const bool vb = sh.n_arr != nullptr;
    const int n = sh.n, nrhs = sh.nrhs;
    cudaStream_t s = queue->stream;
    unsigned long long *stats = (unsigned long long *)(w + L.stats);
    int *count = (int *)(w + L.count);
    int cnt[2] = {0, 0};
    cudaMemcpyAsync(&cnt[0], count, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    if (cnt[0] == 0) return 0;
    double **cA = (double **)(w + L.ca);
    int **cP = (int **)(w + L.cp);
    double **cGB = (double **)(w + L.cx);
    int *csize = vb ? (int *)(w + L.csize) : nullptr;
    double **cA2 = (double **)(w + L.ca2);
    int **cP2 = (int **)(w + L.cp2);
    int *cidx2 = (int *)(w + L.cidx);
    int *cinfo2 = (int *)(w + L.cinfo);
    int *csize2 = vb ? (int *)(w + L.csize2) : nullptr;
    cudaMemsetAsync(count + 1, 0, 2 * sizeof(int), s);
    MLU_LAUNCH(mlu::KC_OTHER, s, ir_compact_adj_kernel<<<batchCount, 256, 0, s>>>(
        sh, dA_array, dipiv_array, dG_array, dGB_array, stats, batchCount, count + 1, cA, cP, cGB,
        csize, cA2, cP2, cidx2, csize2));
    cudaMemcpyAsync(cnt, count + 1, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    magma_int_t rc = 0;
    if (cnt[1] > 0) {
        if (vb)
            rc = vb_run<double>(csize2, csize2, nullptr, n, n, 0, cA2, csize2 + batchCount, cP2,
                                nullptr, nullptr, cinfo2, w + L.vbw, cnt[1], queue, nullptr);
        else
            rc = magma_dgetrf_batched(n, n, cA2, sh.lda, cP2, cinfo2, cnt[1], queue);
        if (rc != 0) return rc;
        MLU_LAUNCH(mlu::KC_OTHER, s, ir_scatter_info_kernel<<<mlu_ceildiv(cnt[1], 256), 256, 0, s>>>(
            cnt[1], cidx2, cinfo2, dinfo_array));
    }
    if (vb)
        return vb_getrs_run<double>(true, csize, csize + batchCount, n, nrhs, cA,
                                    csize + 2 * batchCount, cP, cGB, csize + 3 * batchCount,
                                    cnt[0], queue);
    return magma_dgetrs_batched(MagmaTrans, n, nrhs, cA, sh.lda, cP, cGB, sh.ldx, cnt[0], queue);
}

// Adjoint of a refinement solve: GB = A^{-T} G with the FP32 factors the
// forward call (precision 900, same workspace, same sizes) left in `work`,
// refined in FP64 like the forward solve (residual G - A^T GB); then, when
// dGA is given, GA = -GB X^T.  Matrices whose forward solve fell back
// (iter_fwd < 0: A holds FP64 factors) and, with `fallback`, matrices whose
// adjoint refinement does not converge (A is then factored in FP64 in place,
// info and ipiv overwritten) get an FP64 transposed solve.  `sh` describes A,
// G (ldb) and GB (ldx).
static magma_int_t
ir_run_adjoint(const IrShape &sh, double **dA_array, magma_int_t **dipiv_array, double **dX_array,
               const int *lddx_arr, int lddx, double **dG_array, double **dGB_array,
               double **dGA_array, const int *lddga_arr, int lddga, const int *diter_fwd,
               magma_int_t *dinfo_array, magma_int_t *diter_array, magma_int_t itermax, double tol,
               magma_int_t fallback, void *work, size_t lwork, magma_int_t batchCount,
               magma_queue_t queue)
{
    const bool vb = sh.n_arr != nullptr;
    const int n = sh.n, nrhs = sh.nrhs;
    const IrLayout L = ir_layout(n, nrhs, mlu_max(batchCount, 0), 900, vb);
    if (work == nullptr || lwork < L.total) return MAGMA_ERR_UNKNOWN;   // checked by the callers
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    if (!ir_fits("magma_dxgesv_adjoint", n, nrhs)) return MAGMA_ERR_NOT_SUPPORTED;
    cudaStream_t s = queue->stream;
    char *w = (char *)work;
    unsigned long long *stats = (unsigned long long *)(w + L.stats);
    int *count = (int *)(w + L.count);
    float **As_array = (float **)(w + L.asp);
    double *R = (double *)(w + L.r);
    const int *perm = (const int *)(w + L.perm);

    cudaMemsetAsync(w, 0, L.asp, s);   // stats and counters of this solve; the factors stay
    const dim3 rows_grid((n + IR_ROWS - 1) / IR_ROWS, batchCount);
    MLU_LAUNCH(mlu::KC_IR_INIT, s, ir_init_adj_kernel<<<rows_grid, IR_ROWS, 0, s>>>(
        sh, dA_array, dG_array, dGB_array, R, stats, diter_fwd, diter_array));
    auto solve = [&](int it) {
        correction_solve<true>(sh, As_array, L.ldas, perm, dGB_array, R, stats, diter_array,
                               nullptr, it, tol, nullptr, nullptr, batchCount, s);
    };
    solve(-1);
    residual<true>(sh, dA_array, dG_array, dGB_array, R, stats, 0, batchCount, s);
    for (int it = 0; it < itermax; it++) {
        solve(it);
        residual<true>(sh, dA_array, dG_array, dGB_array, R, stats, (it + 1) & 1, batchCount, s);
    }
    MLU_LAUNCH(mlu::KC_OTHER, s, ir_final_kernel<<<mlu_ceildiv(batchCount, 256), 256, 0, s>>>(
        sh, stats, diter_array, itermax, tol, batchCount, count));
    MLU_CHECK_LAUNCH();

    // FP64 transposed solves for matrices the refinement did not solve (without
    // `fallback`: none, and no synchronisation, so the call can be captured)
    if (fallback) {
        const magma_int_t rc = adjoint_fp64_solves(sh, L, w, dA_array, dipiv_array, dG_array,
                                                   dGB_array, dinfo_array, batchCount, queue);
        if (rc != 0) return rc;
    }
    if (dGA_array) {
        magma_int_t rc;
        if (vb)
            rc = ger_neg_vbatched<double>(sh.n_arr, sh.nrhs_arr, n, dGB_array, sh.ldx_arr,
                                          dX_array, lddx_arr, dGA_array, lddga_arr, batchCount,
                                          queue);
        else
            rc = magmablas_dger_neg_batched(n, nrhs, dGB_array, sh.ldx, dX_array, lddx, dGA_array,
                                            lddga, batchCount, queue);
        if (rc != 0) return rc;
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

// Argument checks of magma_dsgesv_batched_work (positions shifted by argoff),
// then the uniform refinement.
static magma_int_t
ir_driver(const char *name, int argoff, int prec, magma_int_t n, magma_int_t nrhs, double **dA_array,
          magma_int_t ldda, magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
          double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array, magma_int_t *diter_array,
          magma_int_t itermax, double tol, magma_int_t fallback, void *work, size_t *lwork,
          magma_int_t batchCount, magma_queue_t queue, int solver = 920)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0 || nrhs > IR_NRHS_MAX) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (lddb < mlu_max(1, n)) info = -7;
    else if (lddx < mlu_max(1, n)) info = -9;
    else if (itermax < 0) info = -12;
    if (info != 0) {
        magma_xerbla(name, -info + argoff);
        return info - argoff;
    }
    const IrShape sh = {n, nrhs, ldda, lddb, lddx, nullptr, nullptr, nullptr, nullptr, nullptr};
    return ir_run(prec, sh, dA_array, dipiv_array, dB_array, dX_array, dinfo_array, diter_array,
                  itermax, tol, fallback, work, lwork, batchCount, queue, solver);
}

extern "C" magma_int_t
magma_dsgesv_batched_work(magma_int_t n, magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                          magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                          double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                          magma_int_t *diter_array, magma_int_t itermax, double tol,
                          magma_int_t fallback, void *work, size_t *lwork,
                          magma_int_t batchCount, magma_queue_t queue)
{
    return ir_driver(__func__, 0, 900, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb, dX_array,
                     lddx, dinfo_array, diter_array, itermax, tol, fallback, work, lwork,
                     batchCount, queue);
}

extern "C" magma_int_t
magma_dxgesv_batched_work(magma_int_t precision, magma_int_t n, magma_int_t nrhs,
                          double **dA_array, magma_int_t ldda, magma_int_t **dipiv_array,
                          double **dB_array, magma_int_t lddb, double **dX_array,
                          magma_int_t lddx, magma_int_t *dinfo_array, magma_int_t *diter_array,
                          magma_int_t itermax, double tol, magma_int_t fallback, void *work,
                          size_t *lwork, magma_int_t batchCount, magma_queue_t queue)
{
    if (precision != 900 && precision != 905 && precision != 930) {
        magma_xerbla(__func__, 1);
        return -1;
    }
    // argument i of magma_dsgesv_batched_work is argument i+1 here
    return ir_driver(__func__, 1, precision, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                     dX_array, lddx, dinfo_array, diter_array, itermax, tol, fallback, work, lwork,
                     batchCount, queue);
}

extern "C" magma_int_t
magma_dxgesv_gmres_batched_work(magma_int_t precision, magma_int_t solver_type, magma_int_t n,
                                magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                                magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                                double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                                magma_int_t *diter_array, magma_int_t itermax, double tol,
                                magma_int_t fallback, void *work, size_t *lwork,
                                magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (precision != 900 && precision != 905 && precision != 930) info = -1;
    else if (solver_type != 920 && solver_type != 922) info = -2;
    else if (solver_type == 922 && (nrhs < 0 || nrhs > GM_NRHS_MAX)) info = -4;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    // argument i of magma_dsgesv_batched_work is argument i+2 here
    return ir_driver(__func__, 2, precision, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                     dX_array, lddx, dinfo_array, diter_array, itermax, tol, fallback, work, lwork,
                     batchCount, queue, (int)solver_type);
}

// Batched form of magma_dsposv_gpu (src/zcposv_gpu.cpp:134-360): FP32 Cholesky of float(A)
// (lower), FP64 residual, update and stopping rule with FP32 L L^T corrections; the
// iteration codes of magma_dsgesv_batched_work (-3: the FP32 Cholesky found a
// non-positive pivot), and with `fallback` an FP64 magma_dposv_batched of the matrices
// that did not converge (A then holds their FP64 factor).
extern "C" magma_int_t
magma_dsposv_batched_work(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs, double **dA_array,
                          magma_int_t ldda, double **dB_array, magma_int_t lddb,
                          double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                          magma_int_t *diter_array, magma_int_t itermax, double tol,
                          magma_int_t fallback, void *work, size_t *lwork,
                          magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (uplo != MagmaLower) info = -1;           // MagmaUpper: not provided, as the batched potrf
    else if (n < 0) info = -2;
    else if (nrhs < 0 || nrhs > IR_NRHS_MAX) info = -3;
    else if (ldda < mlu_max(1, n)) info = -5;
    else if (lddb < mlu_max(1, n)) info = -7;
    else if (lddx < mlu_max(1, n)) info = -9;
    else if (itermax < 0) info = -12;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    const IrShape sh = {n, nrhs, ldda, lddb, lddx, nullptr, nullptr, nullptr, nullptr, nullptr};
    return ir_run(900, sh, dA_array, nullptr, dB_array, dX_array, dinfo_array, diter_array,
                  itermax, tol, fallback, work, lwork, batchCount, queue, 920, true);
}

extern "C" magma_int_t
magma_dsposv_batched(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs, double **dA_array,
                     magma_int_t ldda, double **dB_array, magma_int_t lddb, double **dX_array,
                     magma_int_t lddx, magma_int_t *dinfo_array, magma_int_t *diter_array,
                     magma_int_t batchCount, magma_queue_t queue)
{
    size_t lwork = 0;
    magma_int_t rc = magma_dsposv_batched_work(uplo, n, nrhs, dA_array, ldda, dB_array, lddb,
                                               dX_array, lddx, dinfo_array, diter_array, 30, 0.0,
                                               1, nullptr, &lwork, batchCount, queue);
    if (rc != 0) return rc;
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    if (queue->work_bytes < lwork) {
        if (queue->work) {
            cudaStreamSynchronize(queue->stream);
            cudaFree(queue->work);
        }
        queue->work = nullptr;
        queue->work_bytes = 0;
        if (mlu::device_malloc(&queue->work, lwork) != cudaSuccess) return MAGMA_ERR_DEVICE_ALLOC;
        queue->work_bytes = lwork;
    }
    return magma_dsposv_batched_work(uplo, n, nrhs, dA_array, ldda, dB_array, lddb, dX_array,
                                     lddx, dinfo_array, diter_array, 30, 0.0, 1, queue->work,
                                     &lwork, batchCount, queue);
}

extern "C" magma_int_t
magma_dsgesv_batched(magma_int_t n, magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                     magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                     double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                     magma_int_t *diter_array, magma_int_t batchCount, magma_queue_t queue)
{
    size_t lwork = 0;
    magma_int_t rc = magma_dsgesv_batched_work(n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                               lddb, dX_array, lddx, dinfo_array, diter_array, 30,
                                               0.0, 1, nullptr, &lwork, batchCount, queue);
    if (rc != 0) return rc;
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    if (queue->work_bytes < lwork) {
        if (queue->work) {
            cudaStreamSynchronize(queue->stream);
            cudaFree(queue->work);
        }
        queue->work = nullptr;
        queue->work_bytes = 0;
        if (mlu::device_malloc(&queue->work, lwork) != cudaSuccess) return MAGMA_ERR_DEVICE_ALLOC;
        queue->work_bytes = lwork;
    }
    return magma_dsgesv_batched_work(n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                     dX_array, lddx, dinfo_array, diter_array, 30, 0.0, 1,
                                     queue->work, &lwork, batchCount, queue);
}

// ---------------------------------------------------------------------------
// Variable-size refinement (no counterpart in the reference).

extern "C" magma_int_t
magma_dxgesv_vbatched_work(magma_int_t precision, magma_int_t *n, magma_int_t *nrhs,
                           magma_int_t max_n, magma_int_t max_nrhs, double **dA_array,
                           magma_int_t *ldda, magma_int_t **dipiv_array, double **dB_array,
                           magma_int_t *lddb, double **dX_array, magma_int_t *lddx,
                           magma_int_t *dinfo_array, magma_int_t *diter_array,
                           magma_int_t itermax, double tol, magma_int_t fallback, void *work,
                           size_t *lwork, magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (precision != 900) info = -1;
    else if (max_n < 0) info = -4;
    else if (max_nrhs < 0 || max_nrhs > IR_NRHS_MAX) info = -5;
    else if (itermax < 0) info = -15;
    else if (lwork == nullptr) info = -19;
    else if (batchCount < 0) info = -20;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    const size_t need = ir_layout(max_n, max_nrhs, batchCount, 900, true).total;
    if (work == nullptr) {          // workspace query
        *lwork = need;
        return 0;
    }
    if (*lwork < need) return -18;
    const IrShape sh = {max_n, max_nrhs, 0, 0, 0, n, nrhs, ldda, lddb, lddx};
    return ir_run(900, sh, dA_array, dipiv_array, dB_array, dX_array, dinfo_array, diter_array,
                  itermax, tol, fallback, work, lwork, batchCount, queue);
}

// ---------------------------------------------------------------------------
// Adjoint of the refinement solve (no counterpart in the reference).

extern "C" magma_int_t
magma_dxgesv_adjoint_batched_work(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                  magma_int_t ldda, magma_int_t **dipiv_array, double **dX_array,
                                  magma_int_t lddx, double **dG_array, magma_int_t lddg,
                                  double **dGB_array, magma_int_t lddgb, double **dGA_array,
                                  magma_int_t lddga, magma_int_t *diter_fwd,
                                  magma_int_t *dinfo_array, magma_int_t *diter_array,
                                  magma_int_t itermax, double tol, magma_int_t fallback,
                                  void *work, size_t lwork, magma_int_t batchCount,
                                  magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0 || nrhs > IR_NRHS_MAX) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (lddx < mlu_max(1, n)) info = -7;
    else if (lddg < mlu_max(1, n)) info = -9;
    else if (lddgb < mlu_max(1, n)) info = -11;
    else if (dGA_array != nullptr && lddga < mlu_max(1, n)) info = -13;
    else if (itermax < 0) info = -17;
    else if (batchCount < 0) info = -22;
    else if (work == nullptr || lwork < ir_layout(n, nrhs, batchCount, 900, false).total) info = -21;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    const IrShape sh = {n, nrhs, ldda, lddg, lddgb, nullptr, nullptr, nullptr, nullptr, nullptr};
    return ir_run_adjoint(sh, dA_array, dipiv_array, dX_array, nullptr, lddx, dG_array, dGB_array,
                          dGA_array, nullptr, lddga, diter_fwd, dinfo_array, diter_array, itermax,
                          tol, fallback, work, lwork, batchCount, queue);
}

extern "C" magma_int_t
magma_dxgesv_adjoint_vbatched_work(magma_int_t *n, magma_int_t *nrhs, magma_int_t max_n,
                                   magma_int_t max_nrhs, double **dA_array, magma_int_t *ldda,
                                   magma_int_t **dipiv_array, double **dX_array, magma_int_t *lddx,
                                   double **dG_array, magma_int_t *lddg, double **dGB_array,
                                   magma_int_t *lddgb, double **dGA_array, magma_int_t *lddga,
                                   magma_int_t *diter_fwd, magma_int_t *dinfo_array,
                                   magma_int_t *diter_array, magma_int_t itermax, double tol,
                                   magma_int_t fallback, void *work, size_t lwork,
                                   magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (max_n < 0) info = -3;
    else if (max_nrhs < 0 || max_nrhs > IR_NRHS_MAX) info = -4;
    else if (itermax < 0) info = -19;
    else if (batchCount < 0) info = -24;
    else if (work == nullptr || lwork < ir_layout(max_n, max_nrhs, batchCount, 900, true).total)
        info = -23;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    const IrShape sh = {max_n, max_nrhs, 0, 0, 0, n, nrhs, ldda, lddg, lddgb};
    return ir_run_adjoint(sh, dA_array, dipiv_array, dX_array, lddx, 0, dG_array, dGB_array,
                          dGA_array, lddga, 0, diter_fwd, dinfo_array, diter_array, itermax, tol,
                          fallback, work, lwork, batchCount, queue);
}
