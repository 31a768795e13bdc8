// solve_core.cuh -- blocked triangular solves on right-hand sides held in
// shared memory, shared by getrs (lu_blocked.cu) and the iterative-refinement
// correction solve (ir.cu).
//
// sB holds NR right-hand sides of length n (column c at sB + c*n).  Triangular
// blocks of 32 rows are solved by warp 0 with shuffles, the remaining rows are
// then updated by all threads; every element receives its updates in the
// order of the CPU oracle (oracle/lu_oracle.c, getrs), so results are
// bit-identical to it.  Must be called by all threads of the block; ends with
// a __syncthreads.  ipiv == nullptr skips the row interchanges (the caller
// has applied them already).
#pragma once
#include "common.cuh"

namespace mlu {

// Warp-level copy of the tb x tb diagonal block at (t0, t0) into sD[r][c]
// (coalesced: lanes run down a column), so that the sequential block solves
// below read shared memory instead of issuing one dependent global load per
// step.  Ends with __syncwarp.
template <typename T>
__device__ __forceinline__ void stage_diag_block(const T *A, int ldda, int t0, int tb,
                                                 T (*sD)[33])
{
    const int lane = threadIdx.x & 31;
#pragma unroll 8
    for (int c = 0; c < 32; c++)
        if (c < tb && lane < tb) sD[lane][c] = A[t0 + lane + (size_t)(t0 + c) * ldda];
    __syncwarp();
}

// The same copy by cp.async (warp 0, one group per lane), so that the next
// block's diagonal arrives while the current one is solved.
template <typename T>
__device__ __forceinline__ void stage_diag_block_async(const T *A, int ldda, int t0, int tb,
                                                       T (*sD)[33])
{
    const int lane = threadIdx.x & 31;
#pragma unroll 8
    for (int c = 0; c < 32; c++)
        if (c < tb && lane < tb) cp_async_elem<sizeof(T)>(&sD[lane][c], A + t0 + lane + (size_t)(t0 + c) * ldda, true);
    cp_async_commit();
}

// PIPE (the refinement's correction solve): in the non-transposed solves the
// next diagonal block is staged by cp.async while the current one is solved
// (two buffers), and every thread loads its first row's 32 coefficients before
// the diagonal solve.  Without PIPE the diagonal block is staged when it is
// needed and the coefficients after it -- one buffer and fewer live registers,
// for the kernels whose occupancy depends on them.
// NR consecutive values from shared memory, 16 bytes at a time (FP32, NR a
// multiple of 4).  The loads are volatile so that the compiler re-reads them per
// row instead of keeping every row's worth in registers.
template <typename T, int NR>
__device__ __forceinline__ void load_row_smem(const T *p, T (&v)[NR])
{
    static_assert(sizeof(T) == 4 && NR % 4 == 0, "FP32 rows of a multiple of four");
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
#pragma unroll
    for (int q = 0; q < NR / 4; q++)
        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n"
                     : "=f"(v[4 * q]), "=f"(v[4 * q + 1]), "=f"(v[4 * q + 2]), "=f"(v[4 * q + 3])
                     : "r"(a + 16 * q)
                     : "memory");
}

template <typename T, bool TRANS, int SOLVE_NR, bool PIPE = false>
__device__ void solve_smem(int n, const T *A, int ldda, const int *ipiv, T *sB, int nr)
{
    __shared__ T sDD[(PIPE && !TRANS) ? 2 : 1][32][33];   // diagonal blocks
    // (PIPE) the diagonal block's solution, right-hand sides contiguous, so that the
    // update below reads all of one row's values in one or two 16-byte loads
    constexpr int YR = (PIPE && !TRANS) ? 32 : 1, YC = (PIPE && !TRANS) ? SOLVE_NR : 1;
    __shared__ __align__(16) T sY[YR][YC];
    T (*sD)[33] = sDD[0];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (!TRANS) {
        if (ipiv != nullptr && tid < nr) {
            T *b = sB + tid * n;
            for (int k = 0; k < n; k++) {
                const int p = ipiv[k] - 1;
                if (p != k) { T t = b[k]; b[k] = b[p]; b[p] = t; }
            }
        }
        __syncthreads();
        // forward: L y = b.  Per 32-row block: warp 0 solves the diagonal block
        // (staged one block ahead by cp.async) while every thread already has
        // the 32 coefficients of its first row below the block in flight; then
        // all threads update the rows below.
        if (PIPE && warp == 0) stage_diag_block_async<T>(A, ldda, 0, min(32, n), sDD[0]);
        for (int t0 = 0, blk = 0; t0 < n; t0 += 32, blk++) {
            const int tb = min(32, n - t0);
            const int i0 = t0 + tb + tid;
            T lv[32];
            if (PIPE && tb == 32 && i0 < n) {
#pragma unroll
                for (int t = 0; t < 32; t++) lv[t] = A[i0 + (size_t)(t0 + t) * ldda];
            }
            if (warp == 0) {
                if (!PIPE) {
                    stage_diag_block<T>(A, ldda, t0, tb, sDD[0]);
                } else if (t0 + 32 < n) {
                    stage_diag_block_async<T>(A, ldda, t0 + 32, min(32, n - t0 - 32), sDD[(blk + 1) & 1]);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
                __syncwarp();
                T (*D)[33] = sDD[PIPE ? (blk & 1) : 0];
                T y[SOLVE_NR];
                const bool v = lane < tb;
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) y[c] = v ? sB[c * n + t0 + lane] : T(0);
                if (PIPE && tb == 32) {
                    // unrolled: the coefficient loads run ahead of the shuffle chain
#pragma unroll
                    for (int t = 0; t < 32; t++) {
                        const T l = D[lane][t];            // L(t0+lane, t0+t)
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++) {
                            const T yt = __shfl_sync(FULL, y[c], t);
                            if (lane > t) y[c] = Prec<T>::fma_(-l, yt, y[c]);
                        }
                    }
                } else {
                    for (int t = 0; t < tb; t++) {
                        const T l = v ? D[lane][t] : T(0);    // L(t0+lane, t0+t)
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++) {
                            const T yt = __shfl_sync(FULL, y[c], t);
                            if (v && lane > t) y[c] = Prec<T>::fma_(-l, yt, y[c]);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) if (v) sB[c * n + t0 + lane] = y[c];
                if (PIPE && v) {
#pragma unroll
                    for (int c = 0; c < SOLVE_NR; c++) sY[lane % YR][c % YC] = y[c];
                }
            }
            __syncthreads();
            for (int i = i0; i < n; i += blockDim.x) {
                T acc[SOLVE_NR];
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) acc[c] = sB[c * n + i];
                if (tb == 32) {
                    // the row's 32 coefficients (with PIPE the first row's are already here)
                    if (!PIPE || i != i0) {
#pragma unroll
                        for (int t = 0; t < 32; t++) lv[t] = A[i + (size_t)(t0 + t) * ldda];
                    }
#pragma unroll
                    for (int t = 0; t < 32; t++) {
                        T yv[SOLVE_NR];
                        if constexpr (PIPE) load_row_smem<T, SOLVE_NR>(&sY[t % YR][0], yv);
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-lv[t], PIPE ? yv[c] : sB[c * n + t0 + t], acc[c]);
                    }
                } else {
                    for (int t = 0; t < tb; t++) {
                        const T l = A[i + (size_t)(t0 + t) * ldda];
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-l, sB[c * n + t0 + t], acc[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) sB[c * n + i] = acc[c];
            }
            __syncthreads();
        }
        // backward: U x = y, the same overlap (blocks from the bottom)
        if (PIPE && warp == 0)
            stage_diag_block_async<T>(A, ldda, max(0, n - 32), n - max(0, n - 32), sDD[0]);
        for (int t1 = n, blk = 0; t1 > 0; t1 -= 32, blk++) {
            const int t0 = max(0, t1 - 32), tb = t1 - t0;
            T uv0[32];
            if (PIPE && tb == 32 && tid < t0) {
#pragma unroll
                for (int t = 0; t < 32; t++) uv0[t] = A[tid + (size_t)(t0 + t) * ldda];
            }
            if (warp == 0) {
                if (!PIPE) {
                    stage_diag_block<T>(A, ldda, t0, tb, sDD[0]);
                } else if (t0 > 0) {
                    const int p0 = max(0, t0 - 32);
                    stage_diag_block_async<T>(A, ldda, p0, t0 - p0, sDD[(blk + 1) & 1]);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
                __syncwarp();
                T (*sD)[33] = sDD[PIPE ? (blk & 1) : 0];
                T y[SOLVE_NR];
                const bool v = lane < tb;
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) y[c] = v ? sB[c * n + t0 + lane] : T(0);
                // lane t holds U(t0+t, t0+t) and its reciprocal, computed in parallel
                const T dl = v ? sD[lane][lane] : T(1);
                const T rl = T(1) / dl;
                if (PIPE && tb == 32) {
                    // unrolled: coefficient loads and the diagonal shuffles run ahead
#pragma unroll
                    for (int t = 31; t >= 0; t--) {
                        const T u = sD[lane][t];           // U(t0+lane, t0+t)
                        const T d = __shfl_sync(FULL, dl, t);
                        const T r = __shfl_sync(FULL, rl, t);
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++) {
                            const T x = rscale(__shfl_sync(FULL, y[c], t), d, r);
                            if (lane == t) y[c] = x;
                            else if (lane < t) y[c] = Prec<T>::fma_(-u, x, y[c]);
                        }
                    }
                } else {
                    for (int t = tb - 1; t >= 0; t--) {
                        const T u = v ? sD[lane][t] : T(0);   // U(t0+lane, t0+t)
                        const T d = __shfl_sync(FULL, dl, t);
                        const T r = __shfl_sync(FULL, rl, t);
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++) {
                            const T x = rscale(__shfl_sync(FULL, y[c], t), d, r);
                            if (lane == t) y[c] = x;
                            else if (v && lane < t) y[c] = Prec<T>::fma_(-u, x, y[c]);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) if (v) sB[c * n + t0 + lane] = y[c];
                if (PIPE && v) {
#pragma unroll
                    for (int c = 0; c < SOLVE_NR; c++) sY[lane % YR][c % YC] = y[c];
                }
            }
            __syncthreads();
            for (int i = tid; i < t0; i += blockDim.x) {
                T acc[SOLVE_NR];
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) acc[c] = sB[c * n + i];
                if (tb == 32) {
                    if (!PIPE || i != tid) {
#pragma unroll
                        for (int t = 0; t < 32; t++) uv0[t] = A[i + (size_t)(t0 + t) * ldda];
                    }
#pragma unroll
                    for (int t = 31; t >= 0; t--) {
                        T yv[SOLVE_NR];
                        if constexpr (PIPE) load_row_smem<T, SOLVE_NR>(&sY[t % YR][0], yv);
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-uv0[t], PIPE ? yv[c] : sB[c * n + t0 + t], acc[c]);
                    }
                } else {
                    for (int t = tb - 1; t >= 0; t--) {
                        const T u = A[i + (size_t)(t0 + t) * ldda];
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-u, sB[c * n + t0 + t], acc[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) sB[c * n + i] = acc[c];
            }
            __syncthreads();
        }
    } else {
        // U^T y = b (forward), U(t,i) = A[t + i*ldda]
        for (int t0 = 0; t0 < n; t0 += 32) {
            const int tb = min(32, n - t0);
            if (warp == 0) {
                T y[SOLVE_NR];
                const bool v = lane < tb;
                stage_diag_block<T>(A, ldda, t0, tb, sD);
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) y[c] = v ? sB[c * n + t0 + lane] : T(0);
                const T dl = v ? sD[lane][lane] : T(1);
                const T rl = T(1) / dl;
                for (int t = 0; t < tb; t++) {
                    const T u = v ? sD[t][lane] : T(0);           // U(t0+t, t0+lane)
                    const T d = __shfl_sync(FULL, dl, t);
                    const T r = __shfl_sync(FULL, rl, t);
#pragma unroll
                    for (int c = 0; c < SOLVE_NR; c++) {
                        const T x = rscale(__shfl_sync(FULL, y[c], t), d, r);
                        if (lane == t) y[c] = x;
                        else if (v && lane > t) y[c] = Prec<T>::fma_(-u, x, y[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) if (v) sB[c * n + t0 + lane] = y[c];
            }
            __syncthreads();
            for (int i = t0 + tb + tid; i < n; i += blockDim.x) {
                T acc[SOLVE_NR];
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) acc[c] = sB[c * n + i];
                if (tb == 32) {
                    T uv[32];
#pragma unroll
                    for (int t = 0; t < 32; t++) uv[t] = A[(size_t)i * ldda + t0 + t];
#pragma unroll
                    for (int t = 0; t < 32; t++)
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-uv[t], sB[c * n + t0 + t], acc[c]);
                } else {
                    for (int t = 0; t < tb; t++) {
                        const T u = A[(size_t)i * ldda + t0 + t];
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-u, sB[c * n + t0 + t], acc[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) sB[c * n + i] = acc[c];
            }
            __syncthreads();
        }
        // L^T x = y (backward), L(t,i) = A[t + i*ldda] for t > i
        for (int t1 = n; t1 > 0; t1 -= 32) {
            const int t0 = max(0, t1 - 32), tb = t1 - t0;
            if (warp == 0) {
                T y[SOLVE_NR];
                const bool v = lane < tb;
                stage_diag_block<T>(A, ldda, t0, tb, sD);
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) y[c] = v ? sB[c * n + t0 + lane] : T(0);
                for (int t = tb - 1; t >= 0; t--) {
                    const T l = v ? sD[t][lane] : T(0);           // L(t0+t, t0+lane)
#pragma unroll
                    for (int c = 0; c < SOLVE_NR; c++) {
                        const T x = __shfl_sync(FULL, y[c], t);
                        if (v && lane < t) y[c] = Prec<T>::fma_(-l, x, y[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) if (v) sB[c * n + t0 + lane] = y[c];
            }
            __syncthreads();
            for (int i = tid; i < t0; i += blockDim.x) {
                T acc[SOLVE_NR];
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) acc[c] = sB[c * n + i];
                if (tb == 32) {
                    T lv[32];
#pragma unroll
                    for (int t = 0; t < 32; t++) lv[t] = A[(size_t)i * ldda + t0 + t];
#pragma unroll
                    for (int t = 31; t >= 0; t--)
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-lv[t], sB[c * n + t0 + t], acc[c]);
                } else {
                    for (int t = tb - 1; t >= 0; t--) {
                        const T l = A[(size_t)i * ldda + t0 + t];
#pragma unroll
                        for (int c = 0; c < SOLVE_NR; c++)
                            acc[c] = Prec<T>::fma_(-l, sB[c * n + t0 + t], acc[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < SOLVE_NR; c++) sB[c * n + i] = acc[c];
            }
            __syncthreads();
        }
        if (ipiv != nullptr && tid < nr) {
            T *b = sB + tid * n;
            for (int k = n - 1; k >= 0; k--) {
                const int p = ipiv[k] - 1;
                if (p != k) { T t = b[k]; b[k] = b[p]; b[p] = t; }
            }
        }
        __syncthreads();
    }
}

}  // namespace mlu
