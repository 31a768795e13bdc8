// lu_blocked.cu -- blocked right-looking LU and blocked solves for n > 32.
//
// Replaces the blocked part of magma_dgetrf_batched (src/zgetrf_batched.cpp:
// 130-203: recursive panel src/zgetrf_panel_batched.cpp:102-196, fused panel
// magmablas/zgetf2_kernels.cu:833-1058, pivot bookkeeping
// magmablas/getrf_setup_pivinfo.cu:59-309, row swaps
// magmablas/zlaswp_batched.cu:48-89, TRSM magmablas/ztrsm_batched_core.cpp,
// trailing update magmablas/zgemm_batched.cpp:50-97 -> cublasDgemmBatched)
// and the n > 32 part of magma_dgetrs_batched (src/zgetrs_batched.cpp:86-181).
//
// One step of panel width ib at column j0 is three launches:
//   panel_kernel      one CTA per matrix: the (m-j0) x ib panel is staged in
//                     shared memory and factored column by column (lazy row
//                     interchange, pivot search on the integer pipes), then
//                     written back in pivoted order with its pivots;
//   swap_trsm_kernel  one CTA per (matrix, 32-column tile) outside the panel:
//                     applies the panel's interchanges to the tile and, right
//                     of the panel, solves L11 U12 = A12 with one thread per
//                     column;
//   gemm_kernel       one CTA per (matrix, 64x64 tile of A22): A22 -= L21 U12,
//                     one accumulator per element seeded with A22 and updated
//                     in increasing k, so the result is bit-identical to the
//                     unblocked elimination order.
// No workspace and no host synchronisation: every call is stream-ordered and
// capturable in a CUDA graph.
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"
#include "solve_core.cuh"

namespace mlu {

constexpr int PANEL_THREADS = PANEL_REGS_THREADS;
constexpr int SWAP_THREADS = 128;

// Per-matrix sizes for a variable-size batch (device arrays, or all null for a
// uniform batch).  The step kernels take this matrix's m, n, ld from them, do
// nothing when the matrix is already factored past column j0, and narrow the
// panel to the matrix's last columns.
struct StepSizes {
    const int *m_arr, *n_arr, *ld_arr;
    __device__ __forceinline__ bool get(int mat, int j0, int &m, int &n, int &ld, int &ib) const
    {
        if (m_arr) {
            m = m_arr[mat];
            n = n_arr[mat];
            ld = ld_arr[mat];
        }
        const int mn = min(m, n);
        if (j0 >= mn) return false;
        ib = min(ib, mn - j0);
        return true;
    }
};

template <typename T, bool NOPIV = false>
__global__ void __launch_bounds__(PANEL_THREADS)
panel_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int **ipiv_array,
             int *info_array, StepSizes vs)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_ipiv[PANEL_NB];
    const int mat = blockIdx.x, tid = threadIdx.x;
    if (!vs.get(mat, j0, m, n, ldda, ib)) {
        if (j0 == 0 && tid == 0) info_array[mat] = 0;    // empty matrix
        return;
    }
    T *A = dA_array[mat] + j0 + (size_t)j0 * ldda;
    const int info_local = panel_factor<T, NOPIV>(m - j0, ib, A, ldda, smem_raw, s_ipiv, j0);
    if (ipiv_array && tid < ib) ipiv_array[mat][j0 + tid] = j0 + s_ipiv[tid] + 1;
    if (tid == 0) {
        if (j0 == 0) info_array[mat] = info_local;
        else if (info_local != 0 && info_array[mat] == 0) info_array[mat] = info_local;
    }
}

// Register-resident panel (pm <= RPT * PANEL_THREADS): one barrier per column;
// dynamic shared memory panel_regs_smem_bytes<T, RPT>().
// two CTAs per SM unless the panel rows alone need more than 64 registers
template <typename T, int RPT, bool NOPIV = false>
__global__ void __launch_bounds__(PANEL_THREADS, (sizeof(T) * RPT * PANEL_NB / 4 > 64) ? 1 : 2)
panel_regs_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int **ipiv_array,
                  int *info_array, StepSizes vs)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_ipiv[PANEL_NB];
    const int mat = blockIdx.x, tid = threadIdx.x;
    if (!vs.get(mat, j0, m, n, ldda, ib)) {
        if (j0 == 0 && tid == 0) info_array[mat] = 0;    // empty matrix
        return;
    }
    T *A = dA_array[mat] + j0 + (size_t)j0 * ldda;
    const int info_local = panel_factor_regs<T, RPT, NOPIV>(m - j0, ib, A, ldda, s_ipiv, j0, smem);
    if (ipiv_array && tid < ib) ipiv_array[mat][j0 + tid] = j0 + s_ipiv[tid] + 1;
    if (tid == 0) {
        if (j0 == 0) info_array[mat] = info_local;
        else if (info_local != 0 && info_array[mat] == 0) info_array[mat] = info_local;
    }
}

// Rows per thread of the register-resident panel for pm rows, 0 when the
// panel is too tall for registers (FP64: 512 rows, FP32: 1024 rows).
template <typename T>
int panel_rows_per_thread(int pm)
{
    if (pm <= PANEL_THREADS) return 1;
    if (pm <= 2 * PANEL_THREADS) return 2;
    if (sizeof(T) == 4 && pm <= 4 * PANEL_THREADS) return 4;
    return 0;
}

// Applies the interchanges of panel [j0, j0+ib) to a SWAP_COLS-column tile
// outside the panel and, for tiles right of the panel, computes
// U12 = L11^{-1} A12 (one thread per column).
constexpr int SWAP_COLS = 64;

template <typename T>
__global__ void __launch_bounds__(SWAP_THREADS)
swap_trsm_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int **ipiv_array,
                 StepSizes vs)
{
    __shared__ int s_row[2 * PANEL_NB], s_src[2 * PANEL_NB], s_cnt;
    __shared__ T s_tmp[2 * PANEL_NB * (SWAP_W + 1)];
    __shared__ T s_rhs[PANEL_NB * SWAP_COLS];
    const int mat = blockIdx.y;
    if (!vs.get(mat, j0, m, n, ldda, ib)) return;
    T *A = dA_array[mat];
    // column tile: left tiles cover [0, j0), right tiles cover [j0+ib, n)
    const int nleft = (j0 + SWAP_COLS - 1) / SWAP_COLS;
    int c0, c1;
    bool right;
    if ((int)blockIdx.x < nleft) {
        c0 = blockIdx.x * SWAP_COLS;
        c1 = min(c0 + SWAP_COLS, j0);
        right = false;
    } else {
        c0 = j0 + ib + (blockIdx.x - nleft) * SWAP_COLS;
        c1 = min(c0 + SWAP_COLS, n);
        right = true;
        if (c0 >= n) return;             // past this matrix's columns
    }
    if (ipiv_array == nullptr) {             // no pivoting: no interchanges
        if (threadIdx.x == 0) s_cnt = 0;
    } else if (threadIdx.x < 32) {
        build_permutation(ipiv_array[mat], j0, ib, s_row, s_src, &s_cnt);
    }
    __syncthreads();
    apply_permutation<T>(A, ldda, c0, c1, s_row, s_src, s_cnt, s_tmp);
    if (right) trsm_l11_smem<T>(A, ldda, j0, ib, c0, c1, s_rhs, SWAP_COLS);
}

// A22 -= L21 * U12 on BM x BN tiles, TM x TN accumulators per thread.
template <typename T, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int tiles_m, StepSizes vs)
{
    __shared__ __align__(16) T sL[PANEL_NB * BM];
    __shared__ __align__(16) T sU[BN * GEMM_LDU];
    const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
    if (!vs.get(blockIdx.y, j0, m, n, ldda, ib)) return;
    if (j0 + ib + tm * BM >= m || j0 + ib + tn * BN >= n) return;   // tile past this matrix
    gemm_tile<T, BM, BN, TM, TN>(dA_array[blockIdx.y], ldda, m, n, j0, ib, j0 + ib + tm * BM,
                                 j0 + ib + tn * BN, sL, sU);
}

// Panel width of the step at column j0 (32, halved while the panel's shared
// memory copy does not fit).
template <typename T>
int blocked_panel_width(int m, int n, int j0)
{
    const int want = min(PANEL_NB, min(m, n) - j0);
    if (panel_rows_per_thread<T>(m - j0) > 0) return want;
    return panel_width<T>(m - j0, want, PANEL_SMEM_MAX);
}

// The panel kernel for panels of rpt rows per thread (0: shared memory).
template <typename T, bool NOPIV>
static void launch_panel(int rpt, int m, int n, int j0, int ib, T **dA, int ldda, int **ipiv,
                         int *info, StepSizes vs, int nb, size_t smem, cudaStream_t s)
{
    if (rpt == 1)
        MLU_LAUNCH(mlu::KC_PANEL, s, panel_regs_kernel<T, 1, NOPIV><<<nb, PANEL_THREADS, smem, s>>>(
            m, n, j0, ib, dA, ldda, ipiv, info, vs));
    else if (rpt == 2)
        MLU_LAUNCH(mlu::KC_PANEL, s, panel_regs_kernel<T, 2, NOPIV><<<nb, PANEL_THREADS, smem, s>>>(
            m, n, j0, ib, dA, ldda, ipiv, info, vs));
    else if (rpt == 4)
        MLU_LAUNCH(mlu::KC_PANEL, s,
                   panel_regs_kernel<T, (sizeof(T) == 4 ? 4 : 2), NOPIV><<<nb, PANEL_THREADS, smem, s>>>(
                       m, n, j0, ib, dA, ldda, ipiv, info, vs));
    else
        MLU_LAUNCH(mlu::KC_PANEL, s, panel_kernel<T, NOPIV><<<nb, PANEL_THREADS, smem, s>>>(
            m, n, j0, ib, dA, ldda, ipiv, info, vs));
}

// One step of the blocked factorisation for every matrix: panel at column j0
// of width ib, interchanges + TRSM, and (when `update`) the trailing update.
// `vsz`: per-matrix sizes of a variable-size batch (m, n = their maxima).
template <typename T>
magma_int_t blocked_getrf_steps_l(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                                  magma_queue_t q, int j0, int ib, bool update,
                                  StepSizes vsz = {nullptr, nullptr, nullptr})
{
    cudaStream_t s = q->stream;
    constexpr int BM = 64, BN = 64, TM = 4, TN = 4;
    static size_t panel_dyn_max = 0;
    if (!panel_dyn_max) {
        panel_dyn_max = min(mlu_allow_dynamic_smem(panel_kernel<T, false>),
                            mlu_allow_dynamic_smem(panel_kernel<T, true>));
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 1, false>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 2, false>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, (sizeof(T) == 4 ? 4 : 2), false>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 1, true>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 2, true>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, (sizeof(T) == 4 ? 4 : 2), true>);
    }
    const int pm = m - j0;
    const int rpt = panel_rows_per_thread<T>(pm);
    const size_t smem = rpt == 1   ? panel_regs_smem_bytes<T, 1>()
                        : rpt == 2 ? panel_regs_smem_bytes<T, 2>()
                        : rpt == 4 ? panel_regs_smem_bytes<T, (sizeof(T) == 4 ? 4 : 2)>()
                                   : panel_smem_bytes<T>(pm, ib);
    if (!rpt && (smem > PANEL_SMEM_MAX || smem > panel_dyn_max))
        return MAGMA_ERR_NOT_SUPPORTED;   // m too large for a shared-memory panel
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        T **dAb = dA + b0;
        int **ipb = ipiv ? ipiv + b0 : nullptr;
        int *infb = info + b0;
        StepSizes vs = vsz;
        if (vs.m_arr) {
            vs.m_arr += b0;
            vs.n_arr += b0;
            vs.ld_arr += b0;
        }
        // panel (one CTA per matrix), then interchanges + TRSM (one CTA per
        // matrix and 64-column tile)
        // no pivot array: LU without pivoting (the diagonal is the pivot)
        if (ipiv == nullptr)
            launch_panel<T, true>(rpt, m, n, j0, ib, dAb, ldda, nullptr, infb, vs, nb, smem, s);
        else
            launch_panel<T, false>(rpt, m, n, j0, ib, dAb, ldda, ipb, infb, vs, nb, smem, s);
        const int ncl = (j0 + SWAP_COLS - 1) / SWAP_COLS;
        const int ncr = (n - j0 - ib + SWAP_COLS - 1) / SWAP_COLS;
        if (ncl + ncr > 0)
            MLU_LAUNCH(mlu::KC_SWAP_TRSM, s, swap_trsm_kernel<T><<<dim3(ncl + ncr, nb), SWAP_THREADS, 0, s>>>(
                m, n, j0, ib, dAb, ldda, ipb, vs));
        const int rm = m - j0 - ib, rn = n - j0 - ib;
        if (update && rm > 0 && rn > 0) {
            const int tiles_m = (rm + BM - 1) / BM, tiles_n = (rn + BN - 1) / BN;
            MLU_LAUNCH(mlu::KC_GEMM, s, gemm_kernel<T, BM, BN, TM, TN><<<dim3(tiles_m * tiles_n, nb),
                                                                            (BM / TM) * (BN / TN), 0, s>>>(
                m, n, j0, ib, dAb, ldda, tiles_m, vs));
        }
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

template <typename T>
magma_int_t blocked_getrf_steps(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                                magma_queue_t q, int j0, int ib, bool update)
{
    return blocked_getrf_steps_l<T>(m, n, dA, ldda, ipiv, info, batch, q, j0, ib, update);
}

template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q)
{
    if (batch <= 0 || m == 0 || n == 0) return MAGMA_SUCCESS;
    const int mn = min(m, n);
    for (int j0 = 0; j0 < mn;) {
        const int ib = blocked_panel_width<T>(m, n, j0);
        const magma_int_t rc = blocked_getrf_steps_l<T>(m, n, dA, ldda, ipiv, info, batch, q, j0,
                                                        ib, true);
        if (rc != 0) return rc;
        j0 += ib;
    }
    return MAGMA_SUCCESS;
}

template int blocked_panel_width<float>(int, int, int);
template magma_int_t blocked_getrf_steps<float>(int, int, float **, int, int **, int *, int,
                                                magma_queue_t, int, int, bool);

// Variable-size batch through the step kernels (several CTAs per matrix and
// step, for batches with large matrices): m, n, ld per matrix on the device,
// max_m / max_n their maxima.  The steps advance by the panel width every
// matrix still has columns at; a matrix whose columns are done leaves each
// launch at once.  Same arithmetic as every other path.
template <typename T>
magma_int_t blocked_getrf_vbatched(const int *m, const int *n, const int *ld, int max_m,
                                   int max_n, T **dA, int **ipiv, int *info, int batch,
                                   magma_queue_t q)
{
    if (batch <= 0 || max_m <= 0 || max_n <= 0) return MAGMA_SUCCESS;
    const int mn = min(max_m, max_n);
    const StepSizes vs = {m, n, ld};
    for (int j0 = 0; j0 < mn;) {
        const int ib = blocked_panel_width<T>(max_m, max_n, j0);
        const magma_int_t rc = blocked_getrf_steps_l<T>(max_m, max_n, dA, 0, ipiv, info, batch, q,
                                                        j0, ib, true, vs);
        if (rc != 0) return rc;
        j0 += ib;
    }
    return MAGMA_SUCCESS;
}
template magma_int_t blocked_getrf_vbatched<double>(const int *, const int *, const int *, int, int,
                                                    double **, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrf_vbatched<float>(const int *, const int *, const int *, int, int,
                                                   float **, int **, int *, int, magma_queue_t);

// ---------------------------------------------------------------------------
// Blocked solves.  One CTA per (matrix, group of SOLVE_NR right-hand sides);
// the right-hand sides live in shared memory.  Triangular blocks of 32 are
// solved by warp 0 with shuffles, the rows below/above are then updated by
// all threads; every element receives its updates in the oracle's order.

constexpr int SOLVE_THREADS = 256;
constexpr int SOLVE_NR = 8;

// One CTA per (matrix, group of NR right-hand sides); NR is 4 or 8 so that a
// call with few right-hand sides does not spend FMAs on padding columns.
template <typename T, bool TRANS, int NR>
__global__ void __launch_bounds__(SOLVE_THREADS)
getrs_kernel(int n, int nrhs, T **dA_array, int ldda, int **ipiv_array, T **dB_array, int lddb)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sB = reinterpret_cast<T *>(smem_raw);   // [NR][n]
    const int tid = threadIdx.x;
    const int mat = blockIdx.y;
    const int c0 = blockIdx.x * NR;
    const int nr = min(NR, nrhs - c0);
    const T *A = dA_array[mat];
    const int *ipiv = ipiv_array ? ipiv_array[mat] : nullptr;   // null: no interchanges
    T *B = dB_array[mat] + (size_t)c0 * lddb;

    for (int e = tid; e < NR * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        sB[c * n + i] = c < nr ? B[i + (size_t)c * lddb] : T(0);
    }
    __syncthreads();
    solve_smem<T, TRANS, NR>(n, A, ldda, ipiv, sB, nr);
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        B[i + (size_t)c * lddb] = sB[c * n + i];
    }
}

template <typename T>
magma_int_t blocked_getrs(bool trans, int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB,
                          int lddb, int batch, magma_queue_t q)
{
    if (batch <= 0 || n == 0 || nrhs == 0) return MAGMA_SUCCESS;
    const int nr = nrhs <= 4 ? 4 : SOLVE_NR;
    const size_t smem = (size_t)nr * n * sizeof(T);
    static size_t dyn_max[2][2] = {{0, 0}, {0, 0}};
    size_t &dm = dyn_max[trans][nr == 4];
    if (!dm) {
        if (trans) dm = nr == 4 ? mlu_allow_dynamic_smem(getrs_kernel<T, true, 4>)
                                : mlu_allow_dynamic_smem(getrs_kernel<T, true, SOLVE_NR>);
        else dm = nr == 4 ? mlu_allow_dynamic_smem(getrs_kernel<T, false, 4>)
                          : mlu_allow_dynamic_smem(getrs_kernel<T, false, SOLVE_NR>);
    }
    if (smem > dm) return MAGMA_ERR_NOT_SUPPORTED;
    // one thread per row up to 256 (at least two warps: warp 0 solves the
    // diagonal blocks while the others wait)
    const int threads = min(SOLVE_THREADS, max(64, (n + 31) / 32 * 32));
    cudaStream_t s = q->stream;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        const dim3 grid((nrhs + nr - 1) / nr, nb);
        T **A = dA + b0, **B = dB + b0;
        int **P = ipiv ? ipiv + b0 : nullptr;
        if (trans && nr == 4)
            MLU_LAUNCH(mlu::KC_GETRS, s, getrs_kernel<T, true, 4><<<grid, threads, smem, s>>>(
                n, nrhs, A, ldda, P, B, lddb));
        else if (trans)
            MLU_LAUNCH(mlu::KC_GETRS, s, getrs_kernel<T, true, SOLVE_NR><<<grid, threads, smem, s>>>(
                n, nrhs, A, ldda, P, B, lddb));
        else if (nr == 4)
            MLU_LAUNCH(mlu::KC_GETRS, s, getrs_kernel<T, false, 4><<<grid, threads, smem, s>>>(
                n, nrhs, A, ldda, P, B, lddb));
        else
            MLU_LAUNCH(mlu::KC_GETRS, s, getrs_kernel<T, false, SOLVE_NR><<<grid, threads, smem, s>>>(
                n, nrhs, A, ldda, P, B, lddb));
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

template magma_int_t blocked_getrf<double>(int, int, double **, int, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrf<float>(int, int, float **, int, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrs<double>(bool, int, int, double **, int, int **, double **, int, int, magma_queue_t);
template magma_int_t blocked_getrs<float>(bool, int, int, float **, int, int **, float **, int, int, magma_queue_t);

}  // namespace mlu
