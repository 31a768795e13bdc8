// getri.cu -- batched inverse from the LU factors, out of place.
//
// Replaces magma_dgetri_outofplace_batched (src/zgetri_outofplace_batched.cpp:
// 82-140), which sets invA = I, solves L then U on column blocks with
// recursive batched TRSMs, and finally swaps columns of invA in reverse pivot
// order (LAPACK dgetri's convention, inv(A) = inv(U) inv(L) P^T).  Here one
// CTA per (matrix, group of NR columns) does it in one pass: the identity
// columns are created in shared memory, solved with L and U by the shared
// triangular-solve routine (solve_core.cuh, no row interchanges), and column
// j of Y = inv(U) inv(L) is written straight to its place in inv(A) = Y P^T:
// column perm[j], where perm is the interchange sequence applied to 0..n-1
// ((P^T b)[i] = b[perm[i]]).  No workspace, no synchronisation.  info_array is
// not written (as in the reference).
#include "common.cuh"
#include "trace.cuh"
#include "solve_core.cuh"

namespace mlu {

constexpr int GETRI_NR = 8;
constexpr int GETRI_THREADS = 256;

template <typename T>
__global__ void __launch_bounds__(GETRI_THREADS)
getri_kernel(int n, T **dA_array, int ldda, int **ipiv_array, T **dInv_array, int lddia)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sB = reinterpret_cast<T *>(smem_raw);                              // [NR][n]
    int *s_perm = reinterpret_cast<int *>(sB + (size_t)GETRI_NR * n);     // [n]
    const int mat = blockIdx.y, tid = threadIdx.x;
    const int j0 = blockIdx.x * GETRI_NR;
    const int nr = min(GETRI_NR, n - j0);
    const int *ipiv = ipiv_array[mat];
    for (int i = tid; i < n; i += blockDim.x) s_perm[i] = i;
    for (int e = tid; e < GETRI_NR * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        sB[e] = (c < nr && i == j0 + c) ? T(1) : T(0);
    }
    __syncthreads();
    if (tid == 0) {
        for (int k = 0; k < n; k++) {
            const int p = ipiv[k] - 1;
            if (p != k) { const int t = s_perm[k]; s_perm[k] = s_perm[p]; s_perm[p] = t; }
        }
    }
    __syncthreads();
    solve_smem<T, false, GETRI_NR>(n, dA_array[mat], ldda, nullptr, sB, nr);
    T *Inv = dInv_array[mat];
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        Inv[i + (size_t)s_perm[j0 + c] * lddia] = sB[c * n + i];
    }
}

template <typename T>
static magma_int_t getri_run(const char *name, magma_int_t n, T **dA_array, magma_int_t ldda,
                             magma_int_t **dipiv_array, T **dinvA_array, magma_int_t lddia,
                             magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (ldda < mlu_max(1, n)) info = -3;
    else if (lddia < mlu_max(1, n)) info = -6;
    else if (batchCount < 0) info = -8;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (n == 0 || batchCount == 0) return 0;
    const size_t smem = (size_t)GETRI_NR * n * sizeof(T) + (size_t)n * sizeof(int);
    static size_t dyn_cache[MLU_MAX_DEVICES];
    const size_t dyn_max = mlu_device_cached(dyn_cache, [] { return mlu_allow_dynamic_smem(getri_kernel<T>); });
    if (smem > dyn_max) return MAGMA_ERR_NOT_SUPPORTED;
    const int threads = min(GETRI_THREADS, max(64, (n + 31) / 32 * 32));
    cudaStream_t s = queue->stream;
    for (int b0 = 0; b0 < batchCount; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batchCount - b0, (int)MLU_MAX_GRID_Y);
        const dim3 grid((n + GETRI_NR - 1) / GETRI_NR, nb);
        MLU_LAUNCH(mlu::KC_GETRS, s, getri_kernel<T><<<grid, threads, smem, s>>>(
            n, dA_array + b0, ldda, dipiv_array + b0, dinvA_array + b0, lddia));
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

}  // namespace mlu

extern "C" magma_int_t magma_dgetri_outofplace_batched(magma_int_t n, double **dA_array,
                                                       magma_int_t ldda, magma_int_t **dipiv_array,
                                                       double **dinvA_array, magma_int_t lddia,
                                                       magma_int_t *info_array,
                                                       magma_int_t batchCount, magma_queue_t queue)
{
    (void)info_array;
    return mlu::getri_run<double>(__func__, n, dA_array, ldda, dipiv_array, dinvA_array, lddia,
                                  batchCount, queue);
}

extern "C" magma_int_t magma_sgetri_outofplace_batched(magma_int_t n, float **dA_array,
                                                       magma_int_t ldda, magma_int_t **dipiv_array,
                                                       float **dinvA_array, magma_int_t lddia,
                                                       magma_int_t *info_array,
                                                       magma_int_t batchCount, magma_queue_t queue)
{
    (void)info_array;
    return mlu::getri_run<float>(__func__, n, dA_array, ldda, dipiv_array, dinvA_array, lddia,
                                 batchCount, queue);
}
