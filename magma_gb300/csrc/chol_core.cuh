// chol_core.cuh -- the batched Cholesky solve in shared memory, shared by
// chol.cu (magma_?potrs_batched) and ir.cu (the corrections of the
// mixed-precision SPD refinement).
#pragma once
#include "common.cuh"

namespace mlu {

// Solves L L^T X = B for NR right-hand sides in shared memory (column c at
// sB + c*n): forward L y = b then backward L^T x = y, blocks of 32 solved by
// warp 0 with shuffles, the rows below/above updated by all threads with the
// block's coefficients prefetched.  y_t = y_t * (1/l_tt) (sfmin rule), then
// y_i = fma(-l_it, y_t, y_i) for i > t; backward x_t = x_t * (1/l_tt), then
// x_i = fma(-l_ti, x_t, x_i) for i < t.
template <typename T, int NR>
__device__ void chol_solve_smem(int n, const T *A, int lda, T *sB)
{
    __shared__ T sD[32][33];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // forward
    for (int t0 = 0; t0 < n; t0 += 32) {
        const int tb = min(32, n - t0);
        if (warp == 0) {
            for (int c = 0; c < 32; c++)
                if (c < tb && lane < tb) sD[lane][c] = A[t0 + lane + (size_t)(t0 + c) * lda];
            __syncwarp();
            const bool v = lane < tb;
            T y[NR];
#pragma unroll
            for (int c = 0; c < NR; c++) y[c] = v ? sB[c * n + t0 + lane] : T(0);
            const T dl = v ? sD[lane][lane] : T(1);
            const T rl = T(1) / dl;
            for (int t = 0; t < tb; t++) {
                const T l = v ? sD[lane][t] : T(0);
                const T d = __shfl_sync(FULL, dl, t), r = __shfl_sync(FULL, rl, t);
#pragma unroll
                for (int c = 0; c < NR; c++) {
                    const T x = rscale(__shfl_sync(FULL, y[c], t), d, r);
                    if (lane == t) y[c] = x;
                    else if (v && lane > t) y[c] = Prec<T>::fma_(-l, x, y[c]);
                }
            }
#pragma unroll
            for (int c = 0; c < NR; c++) if (v) sB[c * n + t0 + lane] = y[c];
        }
        __syncthreads();
        for (int i = t0 + tb + tid; i < n; i += blockDim.x) {
            T acc[NR], l[32];
#pragma unroll
            for (int c = 0; c < NR; c++) acc[c] = sB[c * n + i];
#pragma unroll
            for (int t = 0; t < 32; t++) l[t] = t < tb ? A[i + (size_t)(t0 + t) * lda] : T(0);
#pragma unroll
            for (int t = 0; t < 32; t++)
                if (t < tb)
#pragma unroll
                    for (int c = 0; c < NR; c++)
                        acc[c] = Prec<T>::fma_(-l[t], sB[c * n + t0 + t], acc[c]);
#pragma unroll
            for (int c = 0; c < NR; c++) sB[c * n + i] = acc[c];
        }
        __syncthreads();
    }
    // backward, blocks of 32 from the end
    for (int t1 = n; t1 > 0; t1 -= 32) {
        const int t0 = max(0, t1 - 32), tb = t1 - t0;
        if (warp == 0) {
            for (int c = 0; c < 32; c++)
                if (c < tb && lane < tb) sD[lane][c] = A[t0 + lane + (size_t)(t0 + c) * lda];
            __syncwarp();
            const bool v = lane < tb;
            T y[NR];
#pragma unroll
            for (int c = 0; c < NR; c++) y[c] = v ? sB[c * n + t0 + lane] : T(0);
            const T dl = v ? sD[lane][lane] : T(1);
            const T rl = T(1) / dl;
            for (int t = tb - 1; t >= 0; t--) {
                const T l = v ? sD[t][lane] : T(0);     // L^T(lane, t) = L(t, lane)
                const T d = __shfl_sync(FULL, dl, t), r = __shfl_sync(FULL, rl, t);
#pragma unroll
                for (int c = 0; c < NR; c++) {
                    const T x = rscale(__shfl_sync(FULL, y[c], t), d, r);
                    if (lane == t) y[c] = x;
                    else if (v && lane < t) y[c] = Prec<T>::fma_(-l, x, y[c]);
                }
            }
#pragma unroll
            for (int c = 0; c < NR; c++) if (v) sB[c * n + t0 + lane] = y[c];
        }
        __syncthreads();
        for (int i = tid; i < t0; i += blockDim.x) {
            T acc[NR], l[32];
#pragma unroll
            for (int c = 0; c < NR; c++) acc[c] = sB[c * n + i];
#pragma unroll
            for (int t = 0; t < 32; t++) l[t] = t < tb ? A[t0 + t + (size_t)i * lda] : T(0);
#pragma unroll
            for (int s = 0; s < 32; s++) {
                const int t = 31 - s;
                if (t < tb)
#pragma unroll
                    for (int c = 0; c < NR; c++)
                        acc[c] = Prec<T>::fma_(-l[t], sB[c * n + t0 + t], acc[c]);
            }
#pragma unroll
            for (int c = 0; c < NR; c++) sB[c * n + i] = acc[c];
        }
        __syncthreads();
    }
}

}  // namespace mlu
