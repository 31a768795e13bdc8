// adjoint.cu -- reverse-mode derivative of the batched solve x = A^{-1} b.
//
// No counterpart in the reference (MAGMA has no autograd).  With the forward
// factors P A = L U kept, the adjoint of x = A^{-1} b for an upstream gradient
// gx is
//     gb = A^{-T} gx            (magma_?getrs_batched with MagmaTrans, which
//                                reuses the forward L, U and pivots), and
//     gA = -gb x^T              (rank-nrhs outer product, this file).
// ger_neg_kernel writes gA one CTA per 64x64 tile of one matrix: gb and x
// rows for the tile are staged in shared memory, each thread owns a 4x4
// block, acc = fma(gb_ic, x_jc, acc) for c ascending, gA_ij = -acc.  The
// kernel is bound by the write of gA (8 n^2 bytes per matrix in FP64).
#include "common.cuh"
#include "trace.cuh"

extern "C" magma_int_t magma_dgetrs_batched(magma_trans_t, magma_int_t, magma_int_t, double **,
                                            magma_int_t, magma_int_t **, double **, magma_int_t,
                                            magma_int_t, magma_queue_t);
extern "C" magma_int_t magma_sgetrs_batched(magma_trans_t, magma_int_t, magma_int_t, float **,
                                            magma_int_t, magma_int_t **, float **, magma_int_t,
                                            magma_int_t, magma_queue_t);

namespace mlu {

constexpr int GER_TILE = 64, GER_RMAX = 16;

template <typename T>
__global__ void __launch_bounds__(256)
ger_neg_kernel(int n, int nrhs, T **dG_array, int lddg, T **dX_array, int lddx, T **dGA_array,
               int lddga, int tiles, const int *n_arr, const int *nrhs_arr, const int *lddg_arr,
               const int *lddx_arr, const int *lddga_arr)
{
    __shared__ T sG[GER_RMAX][GER_TILE], sX[GER_RMAX][GER_TILE];
    const int mat = blockIdx.y;
    const int ti = blockIdx.x % tiles, tj = blockIdx.x / tiles;
    const int i0 = ti * GER_TILE, j0 = tj * GER_TILE;
    if (n_arr) {                      // variable sizes: this matrix's own
        n = n_arr[mat];
        nrhs = nrhs_arr[mat];
        lddg = lddg_arr[mat];
        lddx = lddx_arr[mat];
        lddga = lddga_arr[mat];
        if (i0 >= n || j0 >= n) return;
    }
    const T *G = dG_array[mat];
    const T *X = dX_array[mat];
    T *GA = dGA_array[mat];
    const int tid = threadIdx.x;
    const int tr = tid % 16, tc = tid / 16;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = T(0);
    for (int c0 = 0; c0 < nrhs; c0 += GER_RMAX) {
        const int rc = min(GER_RMAX, nrhs - c0);
        __syncthreads();
        for (int e = tid; e < GER_RMAX * GER_TILE; e += 256) {
            const int c = e / GER_TILE, i = e % GER_TILE;
            const bool ok = c < rc;
            sG[c][i] = (ok && i0 + i < n) ? G[i0 + i + (size_t)(c0 + c) * lddg] : T(0);
            sX[c][i] = (ok && j0 + i < n) ? X[j0 + i + (size_t)(c0 + c) * lddx] : T(0);
        }
        __syncthreads();
        for (int c = 0; c < rc; c++) {
            T g[4], x[4];
#pragma unroll
            for (int a = 0; a < 4; a++) g[a] = sG[c][tr * 4 + a];
#pragma unroll
            for (int b = 0; b < 4; b++) x[b] = sX[c][tc * 4 + b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = Prec<T>::fma_(g[a], x[b], acc[a][b]);
        }
    }
#pragma unroll
    for (int b = 0; b < 4; b++) {
        const int j = j0 + tc * 4 + b;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int i = i0 + tr * 4 + a;
            if (i < n && j < n) GA[i + (size_t)j * lddga] = -acc[a][b];
        }
    }
}

template <typename T>
magma_int_t ger_neg(int n, int nrhs, T **dG, int lddg, T **dX, int lddx, T **dGA, int lddga,
                    int batch, magma_queue_t q)
{
    if (n <= 0 || batch <= 0) return 0;
    const int tiles = (n + GER_TILE - 1) / GER_TILE;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        MLU_LAUNCH(mlu::KC_ADJ_GER, q->stream, ger_neg_kernel<T><<<dim3(tiles * tiles, nb), 256, 0, q->stream>>>(
            n, nrhs, dG + b0, lddg, dX + b0, lddx, dGA + b0, lddga, tiles, nullptr, nullptr,
            nullptr, nullptr, nullptr));
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

}  // namespace mlu

template <typename T>
static magma_int_t ger_entry(const char *name, magma_int_t n, magma_int_t nrhs, T **dG,
                             magma_int_t lddg, T **dX, magma_int_t lddx, T **dGA,
                             magma_int_t lddga, magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0) info = -2;
    else if (lddg < mlu_max(1, n)) info = -4;
    else if (lddx < mlu_max(1, n)) info = -6;
    else if (lddga < mlu_max(1, n)) info = -8;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    return mlu::ger_neg<T>(n, nrhs, dG, lddg, dX, lddx, dGA, lddga, batchCount, queue);
}

extern "C" magma_int_t magmablas_dger_neg_batched(magma_int_t n, magma_int_t nrhs,
                                                  double **dG_array, magma_int_t lddg,
                                                  double **dX_array, magma_int_t lddx,
                                                  double **dGA_array, magma_int_t lddga,
                                                  magma_int_t batchCount, magma_queue_t queue)
{
    return ger_entry<double>(__func__, n, nrhs, dG_array, lddg, dX_array, lddx, dGA_array, lddga,
                             batchCount, queue);
}

extern "C" magma_int_t magmablas_sger_neg_batched(magma_int_t n, magma_int_t nrhs,
                                                  float **dG_array, magma_int_t lddg,
                                                  float **dX_array, magma_int_t lddx,
                                                  float **dGA_array, magma_int_t lddga,
                                                  magma_int_t batchCount, magma_queue_t queue)
{
    return ger_entry<float>(__func__, n, nrhs, dG_array, lddg, dX_array, lddx, dGA_array, lddga,
                            batchCount, queue);
}

template <typename T>
static magma_int_t adjoint_entry(const char *name, magma_int_t n, magma_int_t nrhs, T **dLU,
                                 magma_int_t ldda, magma_int_t **dipiv, T **dX, magma_int_t lddx,
                                 T **dG, magma_int_t lddg, T **dGA, magma_int_t lddga,
                                 magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (lddx < mlu_max(1, n)) info = -7;
    else if (lddg < mlu_max(1, n)) info = -9;
    else if (lddga < mlu_max(1, n)) info = -11;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (n == 0 || batchCount <= 0) return 0;
    magma_int_t rc;
    if constexpr (sizeof(T) == 8)
        rc = magma_dgetrs_batched(MagmaTrans, n, nrhs, (double **)dLU, ldda, dipiv, (double **)dG,
                                  lddg, batchCount, queue);
    else
        rc = magma_sgetrs_batched(MagmaTrans, n, nrhs, (float **)dLU, ldda, dipiv, (float **)dG,
                                  lddg, batchCount, queue);
    if (rc != 0) return rc;
    return mlu::ger_neg<T>(n, nrhs, dG, lddg, dX, lddx, dGA, lddga, batchCount, queue);
}

extern "C" magma_int_t magma_dgesv_adjoint_batched(magma_int_t n, magma_int_t nrhs,
                                                   double **dLU_array, magma_int_t ldda,
                                                   magma_int_t **dipiv_array,
                                                   double **dX_array, magma_int_t lddx,
                                                   double **dG_array, magma_int_t lddg,
                                                   double **dGA_array, magma_int_t lddga,
                                                   magma_int_t batchCount, magma_queue_t queue)
{
    return adjoint_entry<double>(__func__, n, nrhs, dLU_array, ldda, dipiv_array, dX_array, lddx,
                                 dG_array, lddg, dGA_array, lddga, batchCount, queue);
}

extern "C" magma_int_t magma_sgesv_adjoint_batched(magma_int_t n, magma_int_t nrhs,
                                                   float **dLU_array, magma_int_t ldda,
                                                   magma_int_t **dipiv_array,
                                                   float **dX_array, magma_int_t lddx,
                                                   float **dG_array, magma_int_t lddg,
                                                   float **dGA_array, magma_int_t lddga,
                                                   magma_int_t batchCount, magma_queue_t queue)
{
    return adjoint_entry<float>(__func__, n, nrhs, dLU_array, ldda, dipiv_array, dX_array, lddx,
                                dG_array, lddg, dGA_array, lddga, batchCount, queue);
}

// ---------------------------------------------------------------------------
// Variable sizes (no counterpart in the reference): GA_k = -G_k X_k^T for
// matrices of order n[k] with nrhs[k] columns; max_n is the largest n[k].

namespace mlu {
template <typename T>
magma_int_t ger_neg_vbatched(const int *n, const int *nrhs, int max_n, T **dG, const int *lddg,
                             T **dX, const int *lddx, T **dGA, const int *lddga, int batch,
                             magma_queue_t q)
{
    if (max_n <= 0 || batch <= 0) return 0;
    const int tiles = (max_n + GER_TILE - 1) / GER_TILE;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        MLU_LAUNCH(mlu::KC_ADJ_GER, q->stream,
                   ger_neg_kernel<T><<<dim3(tiles * tiles, nb), 256, 0, q->stream>>>(
                       max_n, 0, dG + b0, 1, dX + b0, 1, dGA + b0, 1, tiles, n + b0, nrhs + b0,
                       lddg + b0, lddx + b0, lddga + b0));
    }
    MLU_CHECK_LAUNCH();
    return 0;
}
template magma_int_t ger_neg_vbatched<double>(const int *, const int *, int, double **, const int *,
                                              double **, const int *, double **, const int *, int,
                                              magma_queue_t);
}  // namespace mlu

extern "C" magma_int_t magmablas_dger_neg_vbatched(magma_int_t *n, magma_int_t *nrhs,
                                                   magma_int_t max_n, double **dG_array,
                                                   magma_int_t *lddg, double **dX_array,
                                                   magma_int_t *lddx, double **dGA_array,
                                                   magma_int_t *lddga, magma_int_t batchCount,
                                                   magma_queue_t queue)
{
    if (max_n < 0) return -3;
    if (batchCount < 0) return -10;
    return mlu::ger_neg_vbatched<double>(n, nrhs, max_n, dG_array, lddg, dX_array, lddx,
                                         dGA_array, lddga, batchCount, queue);
}
