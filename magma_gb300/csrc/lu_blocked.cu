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
// One step of panel width ib at column j0 is two or three launches:
//   panel_kernel      one CTA per matrix: the (m-j0) x ib panel is staged in
//                     shared memory or registers and factored column by
//                     column (pivot search on the integer pipes), then
//                     written back in pivoted order with its pivots;
//   band_kernel       (FP32, large batches) one CTA per (matrix, 64-column
//                     band right of the panel): the panel's interchanges, the
//                     solve L11 U12 = A12 and A22 -= L21 U12 for every row
//                     tile of the band, U12 kept in shared memory;
//   swap_trsm_kernel  otherwise, one CTA per (matrix, 64-column tile):
//     + gemm_kernel   interchanges and U12, then one CTA per 64x64 tile of
//                     A22 for the update.
// Every element is updated with one accumulator in increasing k, so the
// result is bit-identical to the unblocked elimination order.  The
// interchanges left of each panel are applied after the last step by
// left_swaps_kernel (one coalesced gather per earlier panel) when the matrix
// has at most 1024 rows, else by swap_trsm_kernel in each step.
// No workspace and no host synchronisation: every call is stream-ordered and
// capturable in a CUDA graph.
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"
#include "solve_core.cuh"

namespace mlu {

constexpr int PANEL_THREADS = PANEL_REGS_THREADS;
constexpr int SWAP_THREADS = 128;

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
// NT: threads of the CTA (64 or 128 for panels of at most that many rows: fewer
// warps to synchronise per column, more CTAs per SM).
template <typename T, int RPT, bool NOPIV = false, int NT = PANEL_THREADS>
__global__ void __launch_bounds__(NT, (sizeof(T) * RPT * PANEL_NB / 4 > 64) ? 1 : 2)
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
    const int info_local = panel_factor_regs<T, RPT, NOPIV, NT>(m - j0, ib, A, ldda, s_ipiv, j0, smem);
    if (ipiv_array && tid < ib) ipiv_array[mat][j0 + tid] = j0 + s_ipiv[tid] + 1;
    if (tid == 0) {
        if (j0 == 0) info_array[mat] = info_local;
        else if (info_local != 0 && info_array[mat] == 0) info_array[mat] = info_local;
    }
}

// Rows per thread of the register-resident panel for pm rows, 0 when the
// panel is too tall for registers (FP64: 512 rows, FP32: 1024 rows).
template <typename T>
__host__ __device__ inline int panel_rows_per_thread(int pm)
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
                 StepSizes vs, int with_left, int bj)
{
    __shared__ int s_row[2 * PANEL_NB], s_src[2 * PANEL_NB], s_cnt;
    __shared__ T s_tmp[2 * PANEL_NB * (SWAP_W + 1)];
    __shared__ T s_rhs[PANEL_NB * SWAP_COLS];
    const int mat = blockIdx.y;
    if (!vs.get(mat, j0, m, n, ldda, ib)) return;
    n = block_col_end(bj, m, n);                     // right columns end with the block
    T *A = dA_array[mat];
    // column tile: left tiles cover [0, j0), right tiles cover [j0+ib, n)
    const int nleft = with_left ? (j0 + SWAP_COLS - 1) / SWAP_COLS : 0;
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
gemm_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int tiles_m, StepSizes vs, int bj)
{
    __shared__ __align__(16) T sL[PANEL_NB * BM];
    __shared__ __align__(16) T sU[BN * GEMM_LDU];
    const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
    if (!vs.get(blockIdx.y, j0, m, n, ldda, ib)) return;
    n = block_col_end(bj, m, n);
    if (j0 + ib + tm * BM >= m || j0 + ib + tn * BN >= n) return;   // tile past this matrix
    gemm_tile<T, BM, BN, TM, TN>(dA_array[blockIdx.y], ldda, m, n, j0, ib, j0 + ib + tm * BM,
                                 j0 + ib + tn * BN, sL, sU);
}

// ---------------------------------------------------------------------------
// FP32: the step right of the panel in one launch, one CTA per (matrix,
// BAND_N-column band of columns j0+ib..n).
//   1. the step's interchanges as a table of touched rows (build_permutation,
//      warp 0, while the other loads are in flight);
//   2. the band's original top rows (rows j0..j0+ib) and L11 staged in shared
//      memory, coalesced;
//   3. the interchanged top rows, i.e. U12 before the solve: a top row's new
//      content is an original top row (from shared memory) or a row further
//      down (the only scattered reads: at most ib rows of the band);
//   4. U12 = L11^{-1} U12 in registers, one thread per column, kept in shared
//      memory (k-major) and written back;
//   5. A22 -= L21 U12 in strips of 64 rows x 32 columns, one warp per strip and
//      no block-wide barrier: lane l owns rows l and l+32 of the strip, so
//      every global load and store of A22 is a coalesced 128-byte row segment;
//      the warp stages its strip of L21 in its own shared memory (cp.async),
//      and per k a lane reads its two L21 values (one 8-byte load) and the
//      strip's 32 U12 values (eight broadcast 16-byte loads) for 64 FMAs.  A
//      row that receives an original top row in this step's interchanges
//      (always a top row: each interchange k moves row j0+k, which still holds
//      an original top row, down) takes its value from shared memory, so the
//      interchanges need no scattered writes.
// Per element the same operations, in the same order, as swap_trsm_kernel
// followed by gemm_kernel.  Columns left of the panel are not touched (their
// interchanges are applied by swap_trsm_kernel or, after the last step, by
// left_swaps_kernel).
template <typename T>
__host__ __device__ int blocked_panel_width(int m, int n, int j0);

constexpr int BAND_N = 64;                            // columns per band (per CTA)
constexpr int BAND_THREADS = 256;
constexpr int BAND_WARPS = BAND_THREADS / 32;
constexpr int STRIP_M = 64, STRIP_N = 32;             // one warp's piece of A22
constexpr int BAND_TOP_LD = BAND_N + 1;               // original top rows [k][j]
constexpr int BAND_U_LD = BAND_N + 4;                 // U12 [k][j], 16-byte rows
constexpr int BAND_LOADS = PANEL_NB * BAND_N / BAND_THREADS;   // per thread, 8
static_assert(BAND_LOADS * BAND_THREADS == PANEL_NB * BAND_N, "band staging");
static_assert(STRIP_M == 64 && STRIP_N == 32 && BAND_N == 2 * STRIP_N, "strip layout");

// The band kernel is used for FP32 only.  An FP64 version (one thread per
// column for the solve, 4x4 tiles) was slower than the separate interchange/TRSM
// and update kernels on GB300 (85.6 ms against 79.4 ms for the variable-size
// FP64 solve of 256 matrices of order 128..1024): its solve prologue runs on
// the FP64 pipe while the CTA's other warps wait.
template <typename T>
__host__ __device__ constexpr bool band_used() { return sizeof(T) == 4; }

__host__ __device__ constexpr size_t band_smem_bytes()
{
    return sizeof(float) * ((size_t)PANEL_NB * BAND_U_LD + 2 * (size_t)PANEL_NB * BAND_TOP_LD +
                            (size_t)PANEL_NB * (PANEL_NB + 1) + (size_t)BAND_WARPS * PANEL_NB * STRIP_M);
}

__global__ void __launch_bounds__(BAND_THREADS, 2)
band_kernel(int m, int n, int j0, int ib, float **dA_array, int ldda, int **ipiv_array, StepSizes vs,
            int bj)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sU = reinterpret_cast<float *>(smem_raw);  // [PANEL_NB][BAND_U_LD]: U12, k-major
    float *sTop = sU + PANEL_NB * BAND_U_LD;          // [PANEL_NB][BAND_TOP_LD]: original top rows
    float *sP = sTop + PANEL_NB * BAND_TOP_LD;        // [PANEL_NB][BAND_TOP_LD]: pivot rows below
    float *sL11 = sP + PANEL_NB * BAND_TOP_LD;        // [PANEL_NB][PANEL_NB+1]
    float *sLw = sL11 + PANEL_NB * (PANEL_NB + 1);    // [warp][k][64 rows]: L21 strips
    __shared__ int s_p[PANEL_NB], s_top_src[PANEL_NB], s_top_idx[PANEL_NB];
    __shared__ int s_row[PANEL_NB], s_src[PANEL_NB];
    const int mat = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (!vs.get(mat, j0, m, n, ldda, ib)) return;
    n = block_col_end(bj, m, n);                     // columns right of the panel, up to the block's end
    const int c0 = j0 + ib + blockIdx.x * BAND_N;
    if (c0 >= n) return;                              // past this matrix's columns
    const int w = min(BAND_N, n - c0);
    float *A = dA_array[mat];
    const size_t ld = ldda;
    const int r_first = j0 + ib;
    const int strips_r = m > r_first ? (m - r_first + STRIP_M - 1) / STRIP_M : 0;
    const int halves = (w + STRIP_N - 1) / STRIP_N;
    const int nstrips = strips_r * halves;
    float *myL = sLw + warp * PANEL_NB * STRIP_M;     // [k][lane*2 + h]
    // strip sidx's L21 rows (lane, lane+32) into this warp's buffer
    auto issue_L = [&](int sidx) {
        const int ra = r_first + (sidx / halves) * STRIP_M + lane, rb = ra + 32;
#pragma unroll 4
        for (int k = 0; k < PANEL_NB; k++) {
            const bool ka = k < ib;
            cp_async_elem<4>(myL + k * STRIP_M + lane * 2, ka && ra < m ? A + ra + (size_t)(j0 + k) * ld : A,
                             ka && ra < m);
            cp_async_elem<4>(myL + k * STRIP_M + lane * 2 + 1,
                             ka && rb < m ? A + rb + (size_t)(j0 + k) * ld : A, ka && rb < m);
        }
        cp_async_commit();
    };
    // L21 is final (the panel kernel wrote it): the first strips' copies go first
    if (warp < nstrips) issue_L(warp);
    // pivot targets, the band's original top rows and L11, all in flight together
    int p = j0 + lane;
    if (warp == 0 && ipiv_array != nullptr && lane < ib) p = ipiv_array[mat][j0 + lane] - 1;
    if (warp == 0 && lane < ib && !MLU_BC2(p, 0, m, 1, 201)) p = j0 + lane;
    {
        float v[BAND_LOADS], l[PANEL_NB * PANEL_NB / BAND_THREADS];
#pragma unroll
        for (int u = 0; u < BAND_LOADS; u++) {
            const int e = tid + u * BAND_THREADS, k = e % PANEL_NB, j = e / PANEL_NB;
            v[u] = (k < ib && j < w && MLU_BC2(j0 + k, c0 + j, m, n, 202)) ? A[j0 + k + (size_t)(c0 + j) * ld] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < PANEL_NB * PANEL_NB / BAND_THREADS; u++) {
            const int e = tid + u * BAND_THREADS, i = e % PANEL_NB, t = e / PANEL_NB;
            l[u] = (i < ib && t < ib && MLU_BC2(j0 + i, j0 + t, m, n, 203)) ? A[j0 + i + (size_t)(j0 + t) * ld] : 0.f;
        }
        if (warp == 0) s_p[lane] = p;
#pragma unroll
        for (int u = 0; u < BAND_LOADS; u++) {
            const int e = tid + u * BAND_THREADS, k = e % PANEL_NB, j = e / PANEL_NB;
            sTop[k * BAND_TOP_LD + j] = v[u];
        }
#pragma unroll
        for (int u = 0; u < PANEL_NB * PANEL_NB / BAND_THREADS; u++) {
            const int e = tid + u * BAND_THREADS, i = e % PANEL_NB, t = e / PANEL_NB;
            sL11[i * (PANEL_NB + 1) + t] = l[u];       // L11[i][t]
        }
    }
    __syncthreads();
    {
        // the band's segments of the pivot rows below the top block (the only
        // rows below that can move up), while warp 0 resolves the interchanges
        float v[BAND_LOADS];
#pragma unroll
        for (int u = 0; u < BAND_LOADS; u++) {
            const int e = tid + u * BAND_THREADS, j = e % BAND_N, k = e / BAND_N;
            const int pk = s_p[k];
            v[u] = (k < ib && pk >= r_first && j < w && MLU_BC2(pk, c0 + j, m, n, 204))
                       ? A[pk + (size_t)(c0 + j) * ld] : 0.f;
        }
        if (warp == 0) {
            // The step's interchanges k = 0..ib-1 exchange rows j0+k and p_k in
            // turn; as a gather, new row x = old row tau(x) with
            // tau = P_0 o P_1 o ... o P_ib-1, found by applying the
            // transpositions from the last to the first.  Lane k resolves top
            // row j0+k and pivot row p_k; idx remembers which pivot row (if
            // any) a value is.
            int vt = j0 + lane, it = -1, vp = p, ip = lane;
            for (int k = ib - 1; k >= 0; k--) {
                const int a = j0 + k, pk = __shfl_sync(FULL, p, k);
                if (vt == a) { vt = pk; it = k; } else if (vt == pk) { vt = a; it = -1; }
                if (vp == a) { vp = pk; ip = k; } else if (vp == pk) { vp = a; ip = -1; }
            }
            s_top_src[lane] = vt;
            s_top_idx[lane] = it;
            // a pivot row below the top block always ends up holding an
            // original top row (interchange k moves row j0+k, which still
            // holds an original top row, down)
            s_row[lane] = (lane < ib && p >= r_first) ? p : -1;
            s_src[lane] = vp;
        }
#pragma unroll
        for (int u = 0; u < BAND_LOADS; u++) {
            const int e = tid + u * BAND_THREADS, j = e % BAND_N, k = e / BAND_N;
            sP[k * BAND_TOP_LD + j] = v[u];
        }
    }
    __syncthreads();
    // interchanged top rows into sU[k][j]
#pragma unroll
    for (int u = 0; u < BAND_LOADS; u++) {
        const int e = tid + u * BAND_THREADS, j = e % BAND_N, k = e / BAND_N;
        float x = 0.f;
        if (k < ib) {
            const int src = s_top_src[k], idx = s_top_idx[k];
            if (src < r_first) x = sTop[(src - j0) * BAND_TOP_LD + j];
            else if (idx >= 0) x = sP[idx * BAND_TOP_LD + j];
        }
        sU[k * BAND_U_LD + j] = x;
    }
    __syncthreads();
    {
        // U12 = L11^{-1} U12: four lanes per column, lane q of a group owns rows
        // 8q..8q+7; x_t comes from its owner by a shuffle, then
        // x_i = fma(-l_it, x_t, x_i) for i > t, t ascending
        const int col = tid >> 2, q = tid & 3;
        float x[8];
#pragma unroll
        for (int r = 0; r < 8; r++) x[r] = sU[(q * 8 + r) * BAND_U_LD + col];
#pragma unroll
        for (int t = 0; t < PANEL_NB; t++) {
            if (t < ib) {
                const float xt = __shfl_sync(FULL, x[t % 8], t / 8, 4);
#pragma unroll
                for (int r = 0; r < 8; r++) {
                    const int i = q * 8 + r;
                    if (i > t && i < ib) x[r] = fmaf(-sL11[i * (PANEL_NB + 1) + t], xt, x[r]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < 8; r++) sU[(q * 8 + r) * BAND_U_LD + col] = x[r];
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < BAND_LOADS; u++) {
        const int e = tid + u * BAND_THREADS, k = e % PANEL_NB, j = e / PANEL_NB;
        if (k < ib && j < w && MLU_BC2(j0 + k, c0 + j, m, n, 205))
            A[j0 + k + (size_t)(c0 + j) * ld] = sU[k * BAND_U_LD + j];
    }
    // strips of A22, one warp each
    for (int sidx = warp; sidx < nstrips; sidx += BAND_WARPS) {
        if (sidx != warp) issue_L(sidx);
        const int r0 = r_first + (sidx / halves) * STRIP_M;
        const int cs = (sidx % halves) * STRIP_N;     // first column of the strip in the band
        const int ra = r0 + lane, rb = r0 + lane + 32;
        float acc0[STRIP_N], acc1[STRIP_N];
#pragma unroll
        for (int c = 0; c < STRIP_N; c++) {
            const bool cv = cs + c < w;
            const float *colp = A + (size_t)(c0 + cs + c) * ld;
            acc0[c] = (cv && ra < m && MLU_BC2(ra, c0 + cs + c, m, n, 206)) ? colp[ra] : 0.f;
            acc1[c] = (cv && rb < m && MLU_BC2(rb, c0 + cs + c, m, n, 207)) ? colp[rb] : 0.f;
        }
        // rows of this strip that receive an original top row
        const int prow = s_row[lane];
        unsigned mk = __ballot_sync(FULL, prow >= r0 && prow < r0 + STRIP_M);
        while (mk) {
            const int e = __ffs(mk) - 1;
            mk &= mk - 1;
            const int row = s_row[e], top = s_src[e] - j0;
            if (top >= 0 && top < PANEL_NB) {
                const float *srow = sTop + top * BAND_TOP_LD + cs;
                if (row == ra) {
#pragma unroll
                    for (int c = 0; c < STRIP_N; c++) acc0[c] = srow[c];
                } else if (row == rb) {
#pragma unroll
                    for (int c = 0; c < STRIP_N; c++) acc1[c] = srow[c];
                }
            }
        }
        cp_async_wait<0>();
        __syncwarp();
#pragma unroll 2
        for (int k = 0; k < ib; k++) {
            const float2 lv = *reinterpret_cast<const float2 *>(myL + k * STRIP_M + lane * 2);
            const float4 *urow = reinterpret_cast<const float4 *>(sU + k * BAND_U_LD + cs);
#pragma unroll
            for (int qq = 0; qq < STRIP_N / 4; qq++) {
                const float4 u4 = urow[qq];
                acc0[4 * qq + 0] = fmaf(-lv.x, u4.x, acc0[4 * qq + 0]);
                acc0[4 * qq + 1] = fmaf(-lv.x, u4.y, acc0[4 * qq + 1]);
                acc0[4 * qq + 2] = fmaf(-lv.x, u4.z, acc0[4 * qq + 2]);
                acc0[4 * qq + 3] = fmaf(-lv.x, u4.w, acc0[4 * qq + 3]);
                acc1[4 * qq + 0] = fmaf(-lv.y, u4.x, acc1[4 * qq + 0]);
                acc1[4 * qq + 1] = fmaf(-lv.y, u4.y, acc1[4 * qq + 1]);
                acc1[4 * qq + 2] = fmaf(-lv.y, u4.z, acc1[4 * qq + 2]);
                acc1[4 * qq + 3] = fmaf(-lv.y, u4.w, acc1[4 * qq + 3]);
            }
        }
#pragma unroll
        for (int c = 0; c < STRIP_N; c++) {
            if (cs + c < w) {
                float *colp = A + (size_t)(c0 + cs + c) * ld;
                if (ra < m && MLU_BC2(ra, c0 + cs + c, m, n, 208)) colp[ra] = acc0[c];
                if (rb < m && MLU_BC2(rb, c0 + cs + c, m, n, 209)) colp[rb] = acc1[c];
            }
        }
        __syncwarp();                                 // the buffer is refilled for the next strip
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// Interchanges of the later panels applied, after the last step, to the
// columns of an earlier panel (LAPACK applies them step by step; the columns
// left of the current panel are read by no step, so the order of these moves
// relative to the steps does not matter).  One CTA per (matrix, panel): panel
// [pj0, pj1) takes the interchanges k = pj1 .. mn-1, in that order, on rows
// [pj1, m).  As a gather, new row i = old row tau(i) with
// tau = P_pj1 o P_pj1+1 o ... o P_mn-1 (P_k the transposition (k, ipiv[k]-1)),
// so each thread finds tau for its rows alone by running the transpositions
// from the last to the first.  The columns then move through shared memory a
// chunk at a time, coalesced both ways.  Rows per matrix: at most
// LEFT_ROWS * LEFT_THREADS (2 or 4 rows per thread).
//
// With the two-level blocking (lu_outer.cu) the same gather runs in two parts:
// LEFT_IN_BLOCK right after the panels of a 128-column block, for the block's
// own later interchanges (k < the block's end), so that the block's columns
// are in their final row order when the rank-128 update reads them; and
// LEFT_AFTER_BLOCK after the last step, for the interchanges of the later
// blocks (k >= the block's end).  LEFT_ALL does both at once (one-level
// blocking).  `first`: the panel index of blockIdx.x = 0.
constexpr int LEFT_THREADS = 256;
constexpr int LEFT_DEFER_MAX_M = LEFT_THREADS * 4;
constexpr size_t LEFT_BUF_BYTES = 24 * 1024;
enum LeftMode { LEFT_ALL = 0, LEFT_IN_BLOCK = 1, LEFT_AFTER_BLOCK = 2 };

template <typename T, int LEFT_ROWS>
__global__ void __launch_bounds__(LEFT_THREADS)
left_swaps_kernel(int m, int n, int gm, int gn, T **dA_array, int ldda, int **ipiv_array,
                  StepSizes vs, int first, int mode)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sbuf = reinterpret_cast<T *>(smem_raw);        // [cols][seg]
    __shared__ int s_piv[LEFT_DEFER_MAX_M];
    __shared__ int s_pj[2];
    const int mat = blockIdx.y, tid = threadIdx.x;
    if (tid == 0) {                                   // the panel's columns, as the steps chose them
        int j = 0;
        for (int b = 0; b < first + (int)blockIdx.x; b++) j += blocked_panel_width<T>(gm, gn, j);
        s_pj[0] = j;
        s_pj[1] = j + blocked_panel_width<T>(gm, gn, j);
    }
    __syncthreads();
    const int pj0 = s_pj[0], pj1 = s_pj[1];
    int ib = pj1 - pj0;
    if (!vs.get(mat, pj0, m, n, ldda, ib)) return;
    const int mn = min(m, n);
    // interchanges ks .. ke-1 (rows ks..m-1 move)
    const int bend = block_col_end(pj0 / OUTER_NB * OUTER_NB, m, n);
    const int ks = mode == LEFT_AFTER_BLOCK ? bend : pj1;
    const int ke = mode == LEFT_IN_BLOCK ? min(bend, mn) : mn;
    if (ks >= ke) return;                             // nothing later
    T *A = dA_array[mat];
    const int *ipiv = ipiv_array[mat];
    const int seg = m - ks, nk = ke - ks;
    for (int k = tid; k < nk; k += LEFT_THREADS) {
        s_piv[k] = ipiv[ks + k] - 1;
        if (!MLU_BC2(s_piv[k], 0, m, 1, 301)) s_piv[k] = ks + k;
    }
    __syncthreads();
    int tau[LEFT_ROWS];
#pragma unroll
    for (int u = 0; u < LEFT_ROWS; u++) tau[u] = ks + tid + u * LEFT_THREADS;
    for (int k = ke - 1; k >= ks; k--) {
        const int p = s_piv[k - ks];
#pragma unroll
        for (int u = 0; u < LEFT_ROWS; u++) tau[u] = tau[u] == k ? p : (tau[u] == p ? k : tau[u]);
    }
    const int cols = max(1, min(ib, (int)(LEFT_BUF_BYTES / ((size_t)seg * sizeof(T)))));
    for (int cb = pj0; cb < pj0 + ib; cb += cols) {
        const int wc = min(cols, pj0 + ib - cb);
        const int total = wc * seg;
        for (int e0 = tid; e0 < total; e0 += 8 * LEFT_THREADS) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * LEFT_THREADS;
                if (e < total && MLU_BC2(ks + e % seg, cb + e / seg, m, n, 302))
                    v[u] = A[ks + e % seg + (size_t)(cb + e / seg) * ldda];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * LEFT_THREADS;
                if (e < total) sbuf[e] = v[u];        // [c][i]
            }
        }
        __syncthreads();
        for (int c = 0; c < wc; c++) {
#pragma unroll
            for (int u = 0; u < LEFT_ROWS; u++) {
                const int i = ks + tid + u * LEFT_THREADS, src = tau[u] - ks;
                if (i < m && tau[u] != i && src >= 0 && src < seg && MLU_BC2(i, cb + c, m, n, 303))
                    A[i + (size_t)(cb + c) * ldda] = sbuf[c * seg + src];
            }
        }
        __syncthreads();
    }
}

template <typename T>
constexpr size_t left_swaps_smem_bytes() { return LEFT_BUF_BYTES; }

// Panel width of the step at column j0 (32, halved while the panel's shared
// memory copy does not fit).
template <typename T>
__host__ __device__ int blocked_panel_width(int m, int n, int j0)
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
    const int pm = m - j0;
    if (rpt == 1 && pm <= 64)
        MLU_LAUNCH(mlu::KC_PANEL, s, panel_regs_kernel<T, 1, NOPIV, 64><<<nb, 64, panel_regs_smem_bytes<T, 1, 64>(), s>>>(
            m, n, j0, ib, dA, ldda, ipiv, info, vs));
    else if (rpt == 1 && pm <= 128)
        MLU_LAUNCH(mlu::KC_PANEL, s, panel_regs_kernel<T, 1, NOPIV, 128><<<nb, 128, panel_regs_smem_bytes<T, 1, 128>(), s>>>(
            m, n, j0, ib, dA, ldda, ipiv, info, vs));
    else if (rpt == 1)
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

static int mlu_sm_count()
{
    static size_t cache[MLU_MAX_DEVICES];
    return (int)mlu_device_cached(cache, [] {
        int dev = 0, count = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            count <= 0) {
            cudaGetLastError();
            count = 1;
        }
        return (size_t)count;
    });
}

// One step of the blocked factorisation for every matrix: panel at column j0
// of width ib, interchanges + TRSM, and (when `update`) the trailing update.
// Right of the panel, band_kernel does all three in one launch (FP32, when the
// batch gives it at least two CTAs per SM); otherwise swap_trsm_kernel and
// gemm_kernel (more, smaller CTAs) do.  `defer_left`: the interchanges left of
// the panel are left to left_swaps_kernel after the last step.
// `vsz`: per-matrix sizes of a variable-size batch (m, n = their maxima).
// `bj` >= 0: the step is a panel of the block that starts at column bj, and
// updates only the block's columns (block_col_end).
template <typename T>
magma_int_t blocked_getrf_steps_l(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                                  magma_queue_t q, int j0, int ib, bool update,
                                  StepSizes vsz = {nullptr, nullptr, nullptr},
                                  bool defer_left = false, int bj = -1)
{
    cudaStream_t s = q->stream;
    constexpr int BM = 64, BN = 64, TM = 4, TN = 4;
    static size_t panel_cache[MLU_MAX_DEVICES];
    const size_t panel_dyn_max = mlu_device_cached(panel_cache, [] {
        const size_t v = min(mlu_allow_dynamic_smem(panel_kernel<T, false>),
                             mlu_allow_dynamic_smem(panel_kernel<T, true>));
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 1, false>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 2, false>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, (sizeof(T) == 4 ? 4 : 2), false>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 1, true>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, 2, true>);
        mlu_allow_dynamic_smem(panel_regs_kernel<T, (sizeof(T) == 4 ? 4 : 2), true>);
        if (band_used<T>()) mlu_allow_dynamic_smem(band_kernel);
        return v;
    });
    const FixedChoice tune = fixed_choice(sizeof(T) == 8, m, n);
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
        const int rm = m - j0 - ib, rn = block_col_end(bj, m, n) - j0 - ib;
        const int bands = rn > 0 ? (rn + BAND_N - 1) / BAND_N : 0;
        const bool fused = band_used<T>() && update && bands > 0 &&
                           (long long)bands * nb >= (long long)tune.band_ctas * mlu_sm_count();
        const int ncl = defer_left ? 0 : (j0 + SWAP_COLS - 1) / SWAP_COLS;
        const int ncr = fused ? 0 : (rn + SWAP_COLS - 1) / SWAP_COLS;
        if (ncl + ncr > 0)
            MLU_LAUNCH(mlu::KC_SWAP_TRSM, s, swap_trsm_kernel<T><<<dim3(ncl + ncr, nb), SWAP_THREADS, 0, s>>>(
                m, n, j0, ib, dAb, ldda, ipb, vs, defer_left ? 0 : 1, bj));
        if (fused) {
            MLU_LAUNCH(mlu::KC_GEMM, s, band_kernel<<<dim3(bands, nb), BAND_THREADS, band_smem_bytes(), s>>>(
                m, n, j0, ib, reinterpret_cast<float **>(dAb), ldda, ipb, vs, bj));
        } else if (update && rm > 0 && rn > 0) {
            if (!tune.tile64 || rm <= 32 || rn <= 32) {
                // a thin trailing block: 32 x 32 tiles, so that no FMA of a
                // 64 x 64 tile runs on padding (each costs full FP64 issue slots)
                const int tiles_m = (rm + 31) / 32, tiles_n = (rn + 31) / 32;
                MLU_LAUNCH(mlu::KC_GEMM, s, gemm_kernel<T, 32, 32, 2, 2><<<dim3(tiles_m * tiles_n, nb), 256, 0, s>>>(
                    m, n, j0, ib, dAb, ldda, tiles_m, vs, bj));
            } else {
                const int tiles_m = (rm + BM - 1) / BM, tiles_n = (rn + BN - 1) / BN;
                MLU_LAUNCH(mlu::KC_GEMM, s, gemm_kernel<T, BM, BN, TM, TN><<<dim3(tiles_m * tiles_n, nb),
                                                                                (BM / TM) * (BN / TN), 0, s>>>(
                    m, n, j0, ib, dAb, ldda, tiles_m, vs, bj));
            }
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

// The deferred interchanges left of each panel (left_swaps_kernel), for the
// `panels` panels the steps over max sizes (gm, gn) made.
template <typename T>
static magma_int_t launch_left_swaps(int m, int n, int gm, int gn, T **dA, int ldda, int **ipiv,
                                     int batch, int panels, StepSizes vsz, cudaStream_t s,
                                     int first = 0, int mode = LEFT_ALL)
{
    // panels first .. first+panels-2 (the last panel has no later interchanges
    // of its own block, and LEFT_AFTER_BLOCK is only called with all panels)
    if (panels < 2) return MAGMA_SUCCESS;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        StepSizes vs = vsz;
        if (vs.m_arr) {
            vs.m_arr += b0;
            vs.n_arr += b0;
            vs.ld_arr += b0;
        }
        if (gm <= 2 * LEFT_THREADS)
            MLU_LAUNCH(mlu::KC_SWAP_TRSM, s, left_swaps_kernel<T, 2><<<dim3(panels - 1, nb), LEFT_THREADS,
                                                                       left_swaps_smem_bytes<T>(), s>>>(
                m, n, gm, gn, dA + b0, ldda, ipiv + b0, vs, first, mode));
        else
            MLU_LAUNCH(mlu::KC_SWAP_TRSM, s, left_swaps_kernel<T, 4><<<dim3(panels - 1, nb), LEFT_THREADS,
                                                                       left_swaps_smem_bytes<T>(), s>>>(
                m, n, gm, gn, dA + b0, ldda, ipiv + b0, vs, first, mode));
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

magma_int_t outer_update(int m, int n, int J, float **dA, int ldda, int **ipiv, StepSizes vs,
                         int batch, magma_queue_t q);

// The two-level blocking (lu_outer.cu) serves FP32 matrices of at most
// LEFT_DEFER_MAX_M rows (register panels of width 32, interchanges left of the
// panels deferred) with columns right of a first block.
// (and the tuning table chooses it for the size: tuning.cu)
template <typename T>
static bool outer_blocked_shape(int m, int n)
{
    return sizeof(T) == 4 && m <= LEFT_DEFER_MAX_M && n > OUTER_NB && min(m, n) > PANEL_NB;
}
template <typename T>
static bool outer_blocked(int m, int n)
{
    return outer_blocked_shape<T>(m, n) && fixed_choice(false, m, n).two_level;
}

// Steps of the two-level blocked factorisation: per 128-column block, its
// 32-column panels with updates confined to the block, then one rank-128
// update of everything right of it; the interchanges left of each panel after
// the last step, as in the one-level form.
// `outer`: the update right of each block (nullptr: the FP32 SIMT kernel,
// outer_update); it is called with the block's first column J and `ctx`.
typedef magma_int_t (*OuterUpdateFn)(int J, void *ctx);

template <typename T>
static magma_int_t blocked_getrf_outer(int m, int n, T **dA, int ldda, int **ipiv, int *info,
                                       int batch, magma_queue_t q, StepSizes vs,
                                       OuterUpdateFn outer = nullptr, void *ctx = nullptr)
{
    const int mn = min(m, n);
    int panels = 0;
    for (int J = 0; J < mn; J += OUTER_NB) {
        const int E = block_col_end(J, m, n);
        const int first = panels;
        for (int j0 = J; j0 < E; panels++) {
            const int ib = blocked_panel_width<T>(m, n, j0);
            const magma_int_t rc = blocked_getrf_steps_l<T>(m, n, dA, ldda, ipiv, info, batch, q, j0,
                                                            ib, true, vs, true, J);
            if (rc != 0) return rc;
            j0 += ib;
        }
        // the block's own later interchanges on its earlier panels: L11 and L21
        // in their final row order for the rank-128 update
        if (ipiv != nullptr) {
            const magma_int_t rc = launch_left_swaps<T>(m, n, m, n, dA, ldda, ipiv, batch, panels - first, vs,
                                                        q->stream, first, LEFT_IN_BLOCK);
            if (rc != 0) return rc;
        }
        if constexpr (sizeof(T) == 4) {
            if (E < n || vs.m_arr) {
                const magma_int_t rc = outer ? outer(J, ctx) : outer_update(m, n, J, dA, ldda, ipiv, vs, batch, q);
                if (rc != 0) return rc;
            }
        }
    }
    // the later blocks' interchanges on every block's columns
    if (ipiv != nullptr && mn > OUTER_NB)
        return launch_left_swaps<T>(m, n, m, n, dA, ldda, ipiv, batch, panels, vs, q->stream, 0,
                                    LEFT_AFTER_BLOCK);
    return MAGMA_SUCCESS;
}

template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q)
{
    if (batch <= 0 || m == 0 || n == 0) return MAGMA_SUCCESS;
    if (outer_blocked<T>(m, n))
        return blocked_getrf_outer<T>(m, n, dA, ldda, ipiv, info, batch, q, {nullptr, nullptr, nullptr});
    const int mn = min(m, n);
    const bool defer = ipiv != nullptr && m <= LEFT_DEFER_MAX_M;
    int panels = 0;
    for (int j0 = 0; j0 < mn; panels++) {
        const int ib = blocked_panel_width<T>(m, n, j0);
        const magma_int_t rc = blocked_getrf_steps_l<T>(m, n, dA, ldda, ipiv, info, batch, q, j0,
                                                        ib, true, {nullptr, nullptr, nullptr},
                                                        defer);
        if (rc != 0) return rc;
        j0 += ib;
    }
    if (defer)
        return launch_left_swaps<T>(m, n, m, n, dA, ldda, ipiv, batch, panels,
                                    {nullptr, nullptr, nullptr}, q->stream);
    return MAGMA_SUCCESS;
}

// The two-level FP32 factorisation with a caller-provided update right of each
// block (the tensor-core form, lu_tc.cu), for uniform batches that
// outer_blocked() accepts; MAGMA_ERR_NOT_SUPPORTED otherwise.
magma_int_t blocked_getrf_two_level(int m, int n, float **dA, int ldda, int **ipiv, int *info,
                                    int batch, magma_queue_t q, OuterUpdateFn outer, void *ctx)
{
    if (batch <= 0 || m == 0 || n == 0) return MAGMA_SUCCESS;
    if (!outer_blocked<float>(m, n)) return MAGMA_ERR_NOT_SUPPORTED;
    return blocked_getrf_outer<float>(m, n, dA, ldda, ipiv, info, batch, q, {nullptr, nullptr, nullptr},
                                      outer, ctx);
}
bool two_level_applies(int m, int n) { return outer_blocked<float>(m, n); }
bool two_level_possible(int m, int n) { return outer_blocked_shape<float>(m, n); }

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
    if (outer_blocked<T>(max_m, max_n))
        return blocked_getrf_outer<T>(max_m, max_n, dA, 0, ipiv, info, batch, q, vs);
    const bool defer = ipiv != nullptr && max_m <= LEFT_DEFER_MAX_M;
    int panels = 0;
    for (int j0 = 0; j0 < mn; panels++) {
        const int ib = blocked_panel_width<T>(max_m, max_n, j0);
        const magma_int_t rc = blocked_getrf_steps_l<T>(max_m, max_n, dA, 0, ipiv, info, batch, q,
                                                        j0, ib, true, vs, defer);
        if (rc != 0) return rc;
        j0 += ib;
    }
    if (defer)
        return launch_left_swaps<T>(max_m, max_n, max_m, max_n, dA, 0, ipiv, batch, panels, vs,
                                    q->stream);
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
    static size_t dyn_cache[2][2][MLU_MAX_DEVICES];
    size_t *cache = dyn_cache[trans][nr == 4];
    const size_t dm = mlu_device_cached(cache, [&] {
        if (trans) return nr == 4 ? mlu_allow_dynamic_smem(getrs_kernel<T, true, 4>)
                                  : mlu_allow_dynamic_smem(getrs_kernel<T, true, SOLVE_NR>);
        return nr == 4 ? mlu_allow_dynamic_smem(getrs_kernel<T, false, 4>)
                       : mlu_allow_dynamic_smem(getrs_kernel<T, false, SOLVE_NR>);
    });
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
