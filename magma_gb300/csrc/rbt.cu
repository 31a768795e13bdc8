// rbt.cu -- random butterfly transformation (RBT) and the batched solve
// built on it: A x = b becomes (U^T A V) y = U^T b, solved by LU without
// pivoting, then x = V y.
//
// Replaces magma_dgerbt_batched, magmablas_dprbt_batched,
// magmablas_dprbt_mtv_batched / _mv_batched and magma_dgesv_rbt_batched
// (include/magma_zbatched.h:1001-1045, src/zgesv_rbt_batched.cpp,
// src/zgerbt_batched.cpp, magmablas/zgerbt_func_batched.cu).  The transform
// is a depth-2 recursive butterfly (Parker's RBT): U = U_in U_out with U_out a
// butterfly of order n and U_in = diag(B_1, B_2) two butterflies of orders
// n1 = ceil(n/2) and n - n1; V likewise.  A butterfly of order m with random
// diagonals R, S (its m/2 pairs (i, i + m/2)) is
//     B = (1/sqrt 2) [[R, S], [R, -S]],
// and the last element of an odd-order block is left as is.  The
// random diagonals are the 2n entries of u (for U) and v (for V): the outer
// level uses R = w[0..g), S = w[g..2g) with g = n/2, the inner block starting
// at b0 of order m uses R = w[n+b0 ..), S = w[n+b0+m/2 ..).
// U^T A V is applied one level at a time (inner, then outer), each level in
// one pass over A that transforms 2x2 groups of elements in place; per group
// the column transform is applied first, then the row transform:
//     a' = (c R_j) (a + b), b' = (c S_j) (a - b)      (columns j, j + g)
//     a'' = (c R_i) (a' + c'), c'' = (c S_i) (a' - c') (rows i, i + g)
// with c = 1/sqrt 2 and (c R) one rounded product.  No workspace beyond the
// 2n-entry butterflies; magma_dgerbt_batched and magma_dgesv_rbt_batched copy
// them to the device (and synchronise), as the reference does.
#include "common.cuh"
#include "trace.cuh"

#include <cmath>
#include <mutex>

extern "C" magma_int_t magma_dgetrf_nopiv_batched(magma_int_t, magma_int_t, double **, magma_int_t,
                                                  magma_int_t *, magma_int_t, magma_queue_t);
extern "C" magma_int_t magma_dgetrs_nopiv_batched(magma_trans_t, magma_int_t, magma_int_t,
                                                  double **, magma_int_t, double **, magma_int_t,
                                                  magma_int_t *, magma_int_t, magma_queue_t);

namespace mlu {

constexpr double RBT_C = 0.70710678118654752440;   // 1/sqrt(2), rounded once

// Position of index x in the butterfly blocks of `level` (0 outer, 1 inner):
// block start b0, half g, and whether x is a top index (partner x + g), a
// bottom one, or the unpaired last one of an odd block.
struct RbtBlock {
    int b0, g, m;
};

__host__ __device__ inline RbtBlock rbt_block(int level, int n, int x)
{
    if (level == 0) return {0, n / 2, n};
    const int n1 = (n + 1) / 2;
    return x < n1 ? RbtBlock{0, n1 / 2, n1} : RbtBlock{n1, (n - n1) / 2, n - n1};
}

// representative r of a block starting at b0 of order m: its top indices
// b0 .. b0+m/2-1, then (odd m) the unpaired last index b0+m-1
__host__ __device__ inline int rbt_block_rep(int b0, int m, int r)
{
    return r < m / 2 ? b0 + r : b0 + m - 1;
}

// representatives (top or unpaired indices) of one level: r -> index
__host__ __device__ inline int rbt_rep(int level, int n, int r, int *count)
{
    if (level == 0) {
        *count = (n + 1) / 2;
        return rbt_block_rep(0, n, r);
    }
    const int n1 = (n + 1) / 2, c1 = (n1 + 1) / 2, c2 = (n - n1 + 1) / 2;
    *count = c1 + c2;
    return r < c1 ? rbt_block_rep(0, n1, r) : rbt_block_rep(n1, n - n1, r - c1);
}

// index of the representative's butterfly values (R at w[k], S at w[k + g])
__host__ __device__ inline int rbt_value_base(int level, int n, const RbtBlock &b)
{
    return level == 0 ? 0 : n + b.b0;
}

// One level of U^T A V in place, one thread per pair of representatives.
__global__ void rbt_matrix_kernel(int level, int n, double **dA_array, int lda, const double *du,
                                  const double *dv)
{
    int cnt;
    rbt_rep(level, n, 0, &cnt);
    const long long total = (long long)cnt * cnt;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int ri = rbt_rep(level, n, (int)(e % cnt), &cnt);
    const int cj = rbt_rep(level, n, (int)(e / cnt), &cnt);
    double *A = dA_array[blockIdx.y];
    const RbtBlock rb = rbt_block(level, n, ri), cb = rbt_block(level, n, cj);
    const int ki = ri - rb.b0, kj = cj - cb.b0;
    const bool rpair = ki < rb.g, cpair = kj < cb.g;
    const int ri2 = ri + rb.g, cj2 = cj + cb.g;
    double a = A[ri + (size_t)cj * lda];
    double b = cpair ? A[ri + (size_t)cj2 * lda] : 0.0;
    double c = rpair ? A[ri2 + (size_t)cj * lda] : 0.0;
    double d = (rpair && cpair) ? A[ri2 + (size_t)cj2 * lda] : 0.0;
    if (cpair) {                                     // A V: columns cj, cj2
        const int vb = rbt_value_base(level, n, cb) + kj;
        const double wr = RBT_C * dv[vb], ws = RBT_C * dv[vb + cb.g];
        const double a1 = wr * (a + b), b1 = ws * (a - b);
        const double c1 = wr * (c + d), d1 = ws * (c - d);
        a = a1; b = b1; c = c1; d = d1;
    }
    if (rpair) {                                     // U^T (A V): rows ri, ri2
        const int ub = rbt_value_base(level, n, rb) + ki;
        const double wr = RBT_C * du[ub], ws = RBT_C * du[ub + rb.g];
        const double a1 = wr * (a + c), c1 = ws * (a - c);
        const double b1 = wr * (b + d), d1 = ws * (b - d);
        a = a1; c = c1; b = b1; d = d1;
    }
    A[ri + (size_t)cj * lda] = a;
    if (cpair) A[ri + (size_t)cj2 * lda] = b;
    if (rpair) A[ri2 + (size_t)cj * lda] = c;
    if (rpair && cpair) A[ri2 + (size_t)cj2 * lda] = d;
}

// One level of a butterfly applied to the columns of B (n x nrhs):
// TRANS: B <- W^T B (top = (cR)(x + y), bottom = (cS)(x - y)); else
// B <- W B (top = c (R x + S y), bottom = c (R x - S y)).
template <bool TRANS>
__global__ void rbt_vector_kernel(int level, int n, int nrhs, const double *dw,
                                  double **dB_array, int ldb)
{
    int cnt;
    rbt_rep(level, n, 0, &cnt);
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)cnt * nrhs) return;
    const int ri = rbt_rep(level, n, (int)(e % cnt), &cnt);
    const int col = (int)(e / cnt);
    const RbtBlock rb = rbt_block(level, n, ri);
    const int ki = ri - rb.b0;
    if (ki >= rb.g) return;                          // unpaired: unchanged
    double *B = dB_array[blockIdx.y] + (size_t)col * ldb;
    const int wb = rbt_value_base(level, n, rb) + ki;
    const double R = dw[wb], S = dw[wb + rb.g];
    const double x = B[ri], y = B[ri + rb.g];
    if (TRANS) {
        B[ri] = (RBT_C * R) * (x + y);
        B[ri + rb.g] = (RBT_C * S) * (x - y);
    } else {
        const double p = __dmul_rn(R, x), q = __dmul_rn(S, y);   // rounded, never fused
        B[ri] = RBT_C * (p + q);
        B[ri + rb.g] = RBT_C * (p - q);
    }
}

static void rbt_matrix(int n, double **dA, int lda, const double *du, const double *dv, int batch,
                       cudaStream_t s)
{
    for (int level = 1; level >= 0; level--) {              // inner, then outer
        int cnt;
        rbt_rep(level, n, 0, &cnt);
        const long long total = (long long)cnt * cnt;
        for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
            const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
            MLU_LAUNCH(mlu::KC_OTHER, s, rbt_matrix_kernel<<<dim3((unsigned)((total + 255) / 256), nb), 256, 0, s>>>(
                level, n, dA + b0, lda, du, dv));
        }
    }
}

template <bool TRANS>
static void rbt_vectors(int n, int nrhs, const double *dw, double **dB, int ldb, int batch,
                        cudaStream_t s)
{
    // U^T b: inner level then outer; V y: outer level then inner
    for (int step = 0; step < 2; step++) {
        const int level = TRANS ? 1 - step : step;
        int cnt;
        rbt_rep(level, n, 0, &cnt);
        const long long total = (long long)cnt * nrhs;
        for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
            const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
            MLU_LAUNCH(mlu::KC_OTHER, s, rbt_vector_kernel<TRANS><<<dim3((unsigned)((total + 255) / 256), nb), 256, 0, s>>>(
                level, n, nrhs, dw, dB + b0, ldb));
        }
    }
}

// Butterfly diagonals: exp(r / 10) with r uniform in [-1/2, 1/2) (the
// reference's init_butterfly), from one process-wide splitmix64 stream.
static std::mutex g_rbt_mu;
static unsigned long long g_rbt_state = 0x5eed5eed12345678ull;

static double rbt_uniform()
{
    unsigned long long x = (g_rbt_state += 0x9e3779b97f4a7c15ull);
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

static void init_butterfly(int len, double *u, double *v)
{
    std::lock_guard<std::mutex> lk(g_rbt_mu);
    for (int i = 0; i < len; i++) {
        u[i] = std::exp((rbt_uniform() - 0.5) / 10.0);
        v[i] = std::exp((rbt_uniform() - 0.5) / 10.0);
    }
}

}  // namespace mlu

using namespace mlu;

extern "C" void magmablas_dprbt_batched(magma_int_t n, double **dA_array, magma_int_t ldda,
                                        double *du, double *dv, magma_int_t batchCount,
                                        magma_queue_t queue)
{
    if (n <= 1 || batchCount <= 0) return;
    rbt_matrix(n, dA_array, ldda, du, dv, batchCount, queue->stream);
}

extern "C" void magmablas_dprbt_mtv_batched(magma_int_t n, magma_int_t nrhs, double *du,
                                            double **db_array, magma_int_t lddb,
                                            magma_int_t batchCount, magma_queue_t queue)
{
    if (n <= 1 || nrhs <= 0 || batchCount <= 0) return;
    rbt_vectors<true>(n, nrhs, du, db_array, lddb, batchCount, queue->stream);
}

extern "C" void magmablas_dprbt_mv_batched(magma_int_t n, magma_int_t nrhs, double *dv,
                                           double **db_array, magma_int_t lddb,
                                           magma_int_t batchCount, magma_queue_t queue)
{
    if (n <= 1 || nrhs <= 0 || batchCount <= 0) return;
    rbt_vectors<false>(n, nrhs, dv, db_array, lddb, batchCount, queue->stream);
}

extern "C" magma_int_t magma_dgerbt_batched(magma_bool_t gen, magma_int_t n, magma_int_t nrhs,
                                            double **dA_array, magma_int_t ldda,
                                            double **dB_array, magma_int_t lddb, double *U,
                                            double *V, magma_int_t *info, magma_int_t batchCount,
                                            magma_queue_t queue)
{
    *info = 0;
    if (gen != MagmaTrue && gen != MagmaFalse) *info = -1;
    else if (n < 0) *info = -2;
    else if (nrhs < 0) *info = -3;
    else if (ldda < mlu_max(1, n)) *info = -5;
    else if (lddb < mlu_max(1, n)) *info = -7;
    if (*info != 0) {
        magma_xerbla(__func__, -(*info));
        return *info;
    }
    if (nrhs == 0 || n == 0) return 0;
    if (gen == MagmaTrue) init_butterfly(2 * n, U, V);
    double *d = nullptr;
    if (mlu::device_malloc((void **)&d, 4 * (size_t)n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return *info = MAGMA_ERR_DEVICE_ALLOC;
    }
    double *du = d, *dv = d + 2 * n;
    cudaStream_t s = queue->stream;
    cudaMemcpyAsync(du, U, 2 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dv, V, 2 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (batchCount > 0 && n > 1) {
        rbt_matrix(n, dA_array, ldda, du, dv, batchCount, s);
        rbt_vectors<true>(n, nrhs, du, dB_array, lddb, batchCount, s);
    }
    const bool ok = cudaStreamSynchronize(s) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    cudaFree(d);
    return ok ? 0 : (*info = MAGMA_ERR_UNKNOWN);
}

extern "C" magma_int_t magma_dgesv_rbt_batched(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                               magma_int_t ldda, double **dB_array,
                                               magma_int_t lddb, magma_int_t *dinfo_array,
                                               magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (lddb < mlu_max(1, n)) info = -6;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    if (n == 0 || nrhs == 0) return 0;
    double *hu = (double *)malloc(4 * (size_t)n * sizeof(double));
    if (!hu) return MAGMA_ERR_HOST_ALLOC;
    double *hv = hu + 2 * n;
    magma_int_t rc = magma_dgerbt_batched(MagmaTrue, n, nrhs, dA_array, ldda, dB_array, lddb, hu,
                                          hv, &info, batchCount, queue);
    if (rc == 0) rc = magma_dgetrf_nopiv_batched(n, n, dA_array, ldda, dinfo_array, batchCount,
                                                 queue);
    if (rc == 0) rc = magma_dgetrs_nopiv_batched(MagmaNoTrans, n, nrhs, dA_array, ldda, dB_array,
                                                 lddb, dinfo_array, batchCount, queue);
    double *dv = nullptr;
    if (rc == 0 && n > 1) {
        if (mlu::device_malloc((void **)&dv, 2 * (size_t)n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            rc = MAGMA_ERR_DEVICE_ALLOC;
        } else {
            cudaMemcpyAsync(dv, hv, 2 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                            queue->stream);
            rbt_vectors<false>(n, nrhs, dv, dB_array, lddb, batchCount, queue->stream);
            if (cudaStreamSynchronize(queue->stream) != cudaSuccess) rc = MAGMA_ERR_UNKNOWN;
            cudaFree(dv);
        }
    }
    free(hu);
    return rc;
}
