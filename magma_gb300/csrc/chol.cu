// chol.cu -- batched Cholesky factorisation A = L L^T and solve (lower).
//
// Replaces magma_?potrf_batched, magma_?potrs_batched and magma_?posv_batched
// (include/magma_zbatched.h, src/zpotrf_batched.cpp:96-170,
// src/zpotrs_batched.cpp, src/zposv_batched.cpp:90-150; like the reference,
// only MagmaLower -- MagmaUpper returns -1).  Blocked right-looking with
// 32-column panels, each step three launches over the whole batch:
//   chol_diag_kernel   one warp per matrix factors the 32 x 32 diagonal block
//                      in registers (lane = row): d = a_kk, l_kk = sqrt(d),
//                      the column below scaled by 1/l_kk (LAPACK dpotf2), then
//                      a_it = fma(-l_ik, l_tk, a_it) for i >= t > k;
//   chol_trsm_kernel   one thread per row below the block: the row of L21
//                      from L11 (x_k scaled by 1/l_kk, then
//                      x_t = fma(-x_k, l_tk, x_t) for t > k), rows independent;
//   chol_syrk_kernel   A22 -= L21 L21^T on the 64 x 64 tiles on or below the
//                      diagonal (gemm_tile, lower elements stored).
// Every element is updated in increasing k with one accumulator, so the
// factors are those of the unblocked right-looking algorithm.  A non-positive
// or NaN pivot at column j sets info = j (1-based) and stops that matrix:
// later launches leave it as it is (LAPACK dpotrf stops there too).  The
// strictly upper triangle is never written.  No workspace, no
// synchronisation.
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"
#include "chol_core.cuh"

namespace mlu {

constexpr int CHOL_NB = 32;
constexpr int CHOL_TRSM_THREADS = 128;

template <typename T>
__device__ __forceinline__ T sqrt_(T x);
template <>
__device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float sqrt_<float>(float x) { return sqrtf(x); }

// diagonal block [j0, j0+ib) of every matrix, one warp per matrix
template <typename T>
__global__ void __launch_bounds__(32)
chol_diag_kernel(int n, int j0, int ib, T **dA_array, int lda, int *info)
{
    const int mat = blockIdx.x, lane = threadIdx.x;
    if (j0 > 0 && info[mat] != 0) return;               // failed at an earlier step
    T *A = dA_array[mat] + j0 + (size_t)j0 * lda;
    const bool v = lane < ib;
    T a[CHOL_NB];
#pragma unroll
    for (int t = 0; t < CHOL_NB; t++)
        a[t] = (v && t < ib && t <= lane) ? A[lane + (size_t)t * lda] : T(0);
    int fail = 0;
#pragma unroll
    for (int k = 0; k < CHOL_NB; k++) {
        if (k < ib && fail == 0) {
            const T d = __shfl_sync(FULL, a[k], k);
            if (!(d > T(0))) {
                fail = k + 1;                            // not positive definite (or NaN)
            } else {
                const T s = sqrt_<T>(d), r = T(1) / s;
                if (lane == k) a[k] = s;
                else if (lane > k && v) a[k] = rscale(a[k], s, r);
#pragma unroll
                for (int t = k + 1; t < CHOL_NB; t++) {
                    const T ltk = __shfl_sync(FULL, a[k], t);
                    if (t < ib && v && lane >= t) a[t] = Prec<T>::fma_(-a[k], ltk, a[t]);
                }
            }
        }
    }
    // lower triangle back (the columns a failure left were updated up to it)
#pragma unroll
    for (int t = 0; t < CHOL_NB; t++)
        if (v && t < ib && t <= lane) A[lane + (size_t)t * lda] = a[t];
    if (lane == 0) {
        if (j0 == 0) info[mat] = fail;
        else if (fail) info[mat] = j0 + fail;
    }
}

// rows below the diagonal block: x (row of A21) <- x L11^{-T}, one thread per row
template <typename T>
__global__ void __launch_bounds__(CHOL_TRSM_THREADS)
chol_trsm_kernel(int n, int j0, int ib, T **dA_array, int lda, const int *info)
{
    __shared__ T s_L[CHOL_NB][CHOL_NB + 1];
    __shared__ T s_r[CHOL_NB];
    const int mat = blockIdx.y, tid = threadIdx.x;
    if (info[mat] != 0) return;
    T *A = dA_array[mat];
    for (int e = tid; e < ib * ib; e += CHOL_TRSM_THREADS) {
        const int i = e % ib, t = e / ib;
        s_L[i][t] = A[j0 + i + (size_t)(j0 + t) * lda];
    }
    __syncthreads();
    if (tid < ib) s_r[tid] = T(1) / s_L[tid][tid];
    __syncthreads();
    const int row = j0 + ib + blockIdx.x * CHOL_TRSM_THREADS + tid;
    if (row >= n) return;
    T x[CHOL_NB];
#pragma unroll
    for (int t = 0; t < CHOL_NB; t++) x[t] = t < ib ? A[row + (size_t)(j0 + t) * lda] : T(0);
#pragma unroll
    for (int k = 0; k < CHOL_NB; k++) {
        if (k < ib) {
            x[k] = rscale(x[k], s_L[k][k], s_r[k]);
#pragma unroll
            for (int t = k + 1; t < CHOL_NB; t++)
                if (t < ib) x[t] = Prec<T>::fma_(-x[k], s_L[t][k], x[t]);
        }
    }
#pragma unroll
    for (int t = 0; t < CHOL_NB; t++)
        if (t < ib) A[row + (size_t)(j0 + t) * lda] = x[t];
}

// A22 -= L21 L21^T, lower tiles; see gemm_tile (SYRK)
template <typename T>
__global__ void __launch_bounds__(256)
chol_syrk_kernel(int n, int j0, int ib, T **dA_array, int lda, const int *info, int tiles)
{
    __shared__ __align__(16) T sL[PANEL_NB * 64];
    __shared__ __align__(16) T sU[64 * GEMM_LDU];
    const int tm = blockIdx.x % tiles, tn = blockIdx.x / tiles;
    if (tm < tn || info[blockIdx.y] != 0) return;       // tile above the diagonal, or failed
    gemm_tile<T, 64, 64, 4, 4, true>(dA_array[blockIdx.y], lda, n, n, j0, ib, j0 + ib + tm * 64,
                                     j0 + ib + tn * 64, sL, sU);
}

template <typename T>
magma_int_t chol_factor(int n, T **dA, int lda, int *info, int batch, magma_queue_t q)
{
    cudaStream_t s = q->stream;
    for (int j0 = 0; j0 < n; j0 += CHOL_NB) {
        const int ib = min(CHOL_NB, n - j0), rm = n - j0 - ib;
        for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
            const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
            MLU_LAUNCH(mlu::KC_PANEL, s, chol_diag_kernel<T><<<nb, 32, 0, s>>>(
                n, j0, ib, dA + b0, lda, info + b0));
            if (rm > 0) {
                MLU_LAUNCH(mlu::KC_SWAP_TRSM, s,
                           chol_trsm_kernel<T><<<dim3((rm + CHOL_TRSM_THREADS - 1) / CHOL_TRSM_THREADS, nb),
                                                 CHOL_TRSM_THREADS, 0, s>>>(n, j0, ib, dA + b0, lda,
                                                                            info + b0));
                const int tiles = (rm + 63) / 64;
                MLU_LAUNCH(mlu::KC_GEMM, s, chol_syrk_kernel<T><<<dim3(tiles * tiles, nb), 256, 0, s>>>(
                    n, j0, ib, dA + b0, lda, info + b0, tiles));
            }
        }
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

constexpr int CHOL_NR = 4;

template <typename T>
__global__ void __launch_bounds__(256)
chol_solve_kernel(int n, int nrhs, T **dA_array, int lda, T **dB_array, int ldb)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sB = reinterpret_cast<T *>(smem_raw);
    const int mat = blockIdx.y, tid = threadIdx.x;
    const int c0 = blockIdx.x * CHOL_NR, nr = min(CHOL_NR, nrhs - c0);
    T *B = dB_array[mat] + (size_t)c0 * ldb;
    for (int e = tid; e < CHOL_NR * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        sB[e] = c < nr ? B[i + (size_t)c * ldb] : T(0);
    }
    __syncthreads();
    chol_solve_smem<T, CHOL_NR>(n, dA_array[mat], lda, sB);
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        B[i + (size_t)c * ldb] = sB[c * n + i];
    }
}

template <typename T>
magma_int_t chol_solve(int n, int nrhs, T **dA, int lda, T **dB, int ldb, int batch,
                       magma_queue_t q)
{
    const size_t smem = (size_t)CHOL_NR * n * sizeof(T);
    static size_t dyn_cache[MLU_MAX_DEVICES];
    const size_t dyn_max = mlu_device_cached(dyn_cache, [] { return mlu_allow_dynamic_smem(chol_solve_kernel<T>); });
    if (smem > dyn_max) return MAGMA_ERR_NOT_SUPPORTED;
    const int threads = min(256, max(64, (n + 31) / 32 * 32));
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        MLU_LAUNCH(mlu::KC_GETRS, q->stream,
                   chol_solve_kernel<T><<<dim3((nrhs + CHOL_NR - 1) / CHOL_NR, nb), threads, smem, q->stream>>>(
                       n, nrhs, dA + b0, lda, dB + b0, ldb));
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

}  // namespace mlu

using namespace mlu;

template <typename T>
static magma_int_t potrf(const char *name, magma_uplo_t uplo, magma_int_t n, T **dA_array,
                         magma_int_t ldda, magma_int_t *info_array, magma_int_t batchCount,
                         magma_queue_t queue)
{
    magma_int_t info = 0;
    if (uplo != MagmaLower) info = -1;                   // MagmaUpper: not provided, as in MAGMA
    else if (n < 0) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (batchCount < 0) info = -6;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (n == 0 || batchCount == 0) return 0;
    return chol_factor<T>(n, dA_array, ldda, info_array, batchCount, queue);
}

template <typename T>
static magma_int_t potrs(const char *name, magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                         T **dA_array, magma_int_t ldda, T **dB_array, magma_int_t lddb,
                         magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (uplo != MagmaLower) info = -1;
    else if (n < 0) info = -2;
    else if (nrhs < 0) info = -3;
    else if (ldda < mlu_max(1, n)) info = -5;
    else if (lddb < mlu_max(1, n)) info = -7;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    return chol_solve<T>(n, nrhs, dA_array, ldda, dB_array, lddb, batchCount, queue);
}

#define MLU_CHOL(P, T)                                                                          \
    extern "C" magma_int_t magma_##P##potrf_batched(magma_uplo_t uplo, magma_int_t n,           \
                                                    T **dA_array, magma_int_t ldda,             \
                                                    magma_int_t *info_array,                    \
                                                    magma_int_t batchCount,                     \
                                                    magma_queue_t queue)                        \
    {                                                                                           \
        return potrf<T>(__func__, uplo, n, dA_array, ldda, info_array, batchCount, queue);      \
    }                                                                                           \
    extern "C" magma_int_t magma_##P##potrs_batched(magma_uplo_t uplo, magma_int_t n,           \
                                                    magma_int_t nrhs, T **dA_array,             \
                                                    magma_int_t ldda, T **dB_array,             \
                                                    magma_int_t lddb, magma_int_t batchCount,   \
                                                    magma_queue_t queue)                        \
    {                                                                                           \
        return potrs<T>(__func__, uplo, n, nrhs, dA_array, ldda, dB_array, lddb, batchCount,    \
                        queue);                                                                 \
    }                                                                                           \
    extern "C" magma_int_t magma_##P##posv_batched(magma_uplo_t uplo, magma_int_t n,            \
                                                   magma_int_t nrhs, T **dA_array,              \
                                                   magma_int_t ldda, T **dB_array,              \
                                                   magma_int_t lddb, magma_int_t *dinfo_array,  \
                                                   magma_int_t batchCount, magma_queue_t queue) \
    {                                                                                           \
        magma_int_t info = 0;                                                                   \
        if (uplo != MagmaLower) info = -1;                                                      \
        else if (n < 0) info = -2;                                                              \
        else if (nrhs < 0) info = -3;                                                           \
        else if (ldda < mlu_max(1, n)) info = -5;                                               \
        else if (lddb < mlu_max(1, n)) info = -7;                                               \
        if (info != 0) {                                                                        \
            magma_xerbla(__func__, -info);                                                      \
            return info;                                                                        \
        }                                                                                       \
        if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;                                   \
        magma_int_t rc = chol_factor<T>(n, dA_array, ldda, dinfo_array, batchCount, queue);     \
        if (rc != 0) return rc;                                                                 \
        return chol_solve<T>(n, nrhs, dA_array, ldda, dB_array, lddb, batchCount, queue);       \
    }

MLU_CHOL(d, double)
MLU_CHOL(s, float)

namespace mlu {
// the FP32 factorisation of the mixed-precision SPD refinement (ir.cu)
template magma_int_t chol_factor<float>(int, float **, int, int *, int, magma_queue_t);
}  // namespace mlu
