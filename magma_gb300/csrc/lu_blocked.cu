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
#include "solve_core.cuh"

namespace mlu {

constexpr int PANEL_THREADS = 256;
constexpr int PANEL_NB = 32;
constexpr size_t PANEL_SMEM_MAX = 200 * 1024;

template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS)
panel_kernel(int m, int j0, int ib, T **dA_array, int ldda, int **ipiv_array, int *info_array)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int pm = m - j0;           // panel rows
    const int LDS = ib + 1;
    T *sP = reinterpret_cast<T *>(smem_raw);
    int *sPos = reinterpret_cast<int *>(sP + (size_t)pm * LDS);   // logical position of phys row
    int *sRowAt = sPos + pm;                                        // phys row at logical position
    __shared__ unsigned s_whi[PANEL_THREADS / 32], s_wlo[PANEL_THREADS / 32], s_wpos[PANEL_THREADS / 32];
    __shared__ int s_prow, s_ipiv[PANEL_NB];
    __shared__ T s_piv, s_rcp;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int mat = blockIdx.x;
    T *A = dA_array[mat] + j0 + (size_t)j0 * ldda;

    for (int j = 0; j < ib; j++)
        for (int i = tid; i < pm; i += blockDim.x) sP[i * LDS + j] = A[i + (size_t)j * ldda];
    for (int i = tid; i < pm; i += blockDim.x) { sPos[i] = i; sRowAt[i] = i; }
    int info_local = 0;   // meaningful in thread 0
    __syncthreads();

    for (int k = 0; k < ib; k++) {
        // (A) per-thread, then per-warp arg-max over active rows
        unsigned long long best = 0ull;
        unsigned bpos = 0xffffffffu;
        for (int i = tid; i < pm; i += blockDim.x) {
            const int p = sPos[i];
            if (p >= k) {
                const T v = sP[i * LDS + k];
                unsigned long long mag = Prec<T>::absbits(v);
                if (Prec<T>::isnan_(v)) mag = (p == k) ? 0x7fffffffffffffffull : 0ull;
                const unsigned long long key = mag | 0x8000000000000000ull;
                if (key > best || (key == best && (unsigned)p < bpos)) { best = key; bpos = p; }
            }
        }
        {
            const unsigned hi = (unsigned)(best >> 32), lo = (unsigned)best;
            const unsigned mhi = __reduce_max_sync(FULL, hi);
            const unsigned mlo = __reduce_max_sync(FULL, hi == mhi ? lo : 0u);
            const bool cand = hi == mhi && lo == mlo;
            const unsigned wpos = __reduce_min_sync(FULL, cand ? bpos : 0xffffffffu);
            if (lane == 0) { s_whi[warp] = mhi; s_wlo[warp] = mlo; s_wpos[warp] = wpos; }
        }
        __syncthreads();
        // (B) warp 0 combines the warp winners and updates the row maps
        if (warp == 0) {
            const unsigned hi = lane < nwarps ? s_whi[lane] : 0u;
            const unsigned lo = lane < nwarps ? s_wlo[lane] : 0u;
            const unsigned ps = lane < nwarps ? s_wpos[lane] : 0xffffffffu;
            const unsigned mhi = __reduce_max_sync(FULL, hi);
            const unsigned mlo = __reduce_max_sync(FULL, hi == mhi ? lo : 0u);
            const unsigned P = __reduce_min_sync(FULL, (hi == mhi && lo == mlo) ? ps : 0xffffffffu);
            if (lane == 0) {
                const int prow = sRowAt[P];
                const int qrow = sRowAt[k];
                const T piv = sP[prow * LDS + k];
                sPos[prow] = k;
                sRowAt[k] = prow;
                if (qrow != prow) { sPos[qrow] = P; sRowAt[P] = qrow; }
                s_prow = prow;
                s_piv = piv;
                s_rcp = T(1) / piv;
                s_ipiv[k] = (int)P;
                if (!Prec<T>::nonzero(piv) && info_local == 0) info_local = j0 + k + 1;
            }
        }
        __syncthreads();
        // (C) scale the column and update the rest of the panel, own rows only
        const int prow = s_prow;
        const T piv = s_piv, r = s_rcp;
        const bool nz = Prec<T>::nonzero(piv);
        for (int i = tid; i < pm; i += blockDim.x) {
            if (sPos[i] > k) {
                T *row = sP + i * LDS;
                const T v = row[k];
                const T l = nz ? rscale(v, piv, r) : v;
                row[k] = l;
                const T *prw = sP + prow * LDS;
                for (int j = k + 1; j < ib; j++) row[j] = Prec<T>::fma_(-l, prw[j], row[j]);
            }
        }
    }
    __syncthreads();
    // write back in pivoted order
    for (int j = 0; j < ib; j++)
        for (int i = tid; i < pm; i += blockDim.x) A[sPos[i] + (size_t)j * ldda] = sP[i * LDS + j];
    if (tid < ib) ipiv_array[mat][j0 + tid] = j0 + s_ipiv[tid] + 1;
    if (tid == 0) {
        if (j0 == 0) info_array[mat] = info_local;
        else if (info_local != 0 && info_array[mat] == 0) info_array[mat] = info_local;
    }
}

// Applies the interchanges of panel [j0, j0+ib) to a 32-column tile outside
// the panel and, for tiles right of the panel, computes U12 = L11^{-1} A12.
constexpr int SWAP_W = 32;
constexpr int SWAP_THREADS = 128;

template <typename T>
__global__ void __launch_bounds__(SWAP_THREADS)
swap_trsm_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int **ipiv_array)
{
    __shared__ int s_row[2 * PANEL_NB], s_src[2 * PANEL_NB];
    __shared__ int s_cnt;
    __shared__ T s_tmp[2 * PANEL_NB][SWAP_W + 1];
    __shared__ T s_L[PANEL_NB][PANEL_NB + 1];
    const int tid = threadIdx.x, lane = tid & 31;
    const int mat = blockIdx.y;
    T *A = dA_array[mat];
    const int *ipiv = ipiv_array[mat];

    // column tile: left tiles cover [0, j0), right tiles cover [j0+ib, n)
    const int nleft = (j0 + SWAP_W - 1) / SWAP_W;
    int c0, c1;
    bool right;
    if ((int)blockIdx.x < nleft) { c0 = blockIdx.x * SWAP_W; c1 = min(c0 + SWAP_W, j0); right = false; }
    else { c0 = j0 + ib + (blockIdx.x - nleft) * SWAP_W; c1 = min(c0 + SWAP_W, n); right = true; }
    const int w = c1 - c0;

    // compound permutation of the ib sequential interchanges, built by warp 0:
    // s_row[e] is a touched row, s_src[e] the row whose content ends up there
    if (tid < 32) {
        int cnt = 0;
        int r0 = -1, r1 = -1, s0 = -1, s1 = -1;   // lane's entries lane and lane+32
        for (int k = 0; k < ib; k++) {
            const int a = j0 + k, b = ipiv[j0 + k] - 1;
            if (a == b) continue;
            unsigned fa0 = __ballot_sync(FULL, r0 == a), fa1 = __ballot_sync(FULL, r1 == a);
            int ia = fa0 ? __ffs(fa0) - 1 : (fa1 ? 32 + __ffs(fa1) - 1 : -1);
            if (ia < 0) {
                ia = cnt++;
                if (lane == (ia & 31)) { if (ia < 32) { r0 = a; s0 = a; } else { r1 = a; s1 = a; } }
            }
            unsigned fb0 = __ballot_sync(FULL, r0 == b), fb1 = __ballot_sync(FULL, r1 == b);
            int ibb = fb0 ? __ffs(fb0) - 1 : (fb1 ? 32 + __ffs(fb1) - 1 : -1);
            if (ibb < 0) {
                ibb = cnt++;
                if (lane == (ibb & 31)) { if (ibb < 32) { r0 = b; s0 = b; } else { r1 = b; s1 = b; } }
            }
            // swap contents of entries ia and ibb
            const int va = __shfl_sync(FULL, ia < 32 ? s0 : s1, ia & 31);
            const int vb = __shfl_sync(FULL, ibb < 32 ? s0 : s1, ibb & 31);
            if (lane == (ia & 31)) { if (ia < 32) s0 = vb; else s1 = vb; }
            if (lane == (ibb & 31)) { if (ibb < 32) s0 = va; else s1 = va; }
        }
        s_row[lane] = r0; s_src[lane] = s0;
        s_row[lane + 32] = r1; s_src[lane + 32] = s1;
        if (lane == 0) s_cnt = cnt;
    }
    __syncthreads();
    const int cnt = s_cnt;
    // gather all touched rows of the tile, then scatter
    for (int e = tid; e < cnt * SWAP_W; e += blockDim.x) {
        const int pr = e / SWAP_W, c = e % SWAP_W;
        if (c < w) s_tmp[pr][c] = A[s_src[pr] + (size_t)(c0 + c) * ldda];
    }
    __syncthreads();
    for (int e = tid; e < cnt * SWAP_W; e += blockDim.x) {
        const int pr = e / SWAP_W, c = e % SWAP_W;
        if (c < w) A[s_row[pr] + (size_t)(c0 + c) * ldda] = s_tmp[pr][c];
    }
    if (!right) return;
    // L11 (unit lower, ib x ib) to shared memory
    for (int e = tid; e < ib * ib; e += blockDim.x) {
        const int i = e % ib, t = e / ib;
        s_L[i][t] = A[j0 + i + (size_t)(j0 + t) * ldda];
    }
    __syncthreads();
    if (tid < w) {
        T *col = A + j0 + (size_t)(c0 + tid) * ldda;
        T u[PANEL_NB];
#pragma unroll
        for (int i = 0; i < PANEL_NB; i++) u[i] = i < ib ? col[i] : T(0);
#pragma unroll
        for (int t = 0; t < PANEL_NB; t++) {
            if (t >= ib) break;
#pragma unroll
            for (int i = t + 1; i < PANEL_NB; i++)
                if (i < ib) u[i] = Prec<T>::fma_(-s_L[i][t], u[t], u[i]);
        }
#pragma unroll
        for (int i = 0; i < PANEL_NB; i++) if (i < ib) col[i] = u[i];
    }
}

// A22 -= L21 * U12 on BM x BN tiles, TM x TN accumulators per thread.
template <typename T, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_kernel(int m, int n, int j0, int ib, T **dA_array, int ldda, int tiles_m)
{
    constexpr int NT = (BM / TM) * (BN / TN);
    __shared__ __align__(16) T sL[PANEL_NB][BM];
    __shared__ __align__(16) T sU[PANEL_NB][BN];
    const int tid = threadIdx.x;
    const int mat = blockIdx.y;
    const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
    const int r0 = j0 + ib + tm * BM;   // first row of the tile
    const int c0 = j0 + ib + tn * BN;   // first column of the tile
    T *A = dA_array[mat];

    for (int e = tid; e < ib * BM; e += NT) {
        const int i = e % BM, k = e / BM;
        sL[k][i] = (r0 + i < m) ? A[r0 + i + (size_t)(j0 + k) * ldda] : T(0);
    }
    for (int e = tid; e < ib * BN; e += NT) {
        const int k = e % ib, j = e / ib;
        sU[k][j] = (c0 + j < n) ? A[j0 + k + (size_t)(c0 + j) * ldda] : T(0);
    }
    const int tr = tid % (BM / TM), tc = tid / (BM / TM);
    T acc[TM][TN];
#pragma unroll
    for (int b = 0; b < TN; b++) {
        const int c = c0 + tc * TN + b;
#pragma unroll
        for (int a = 0; a < TM; a++) {
            const int r = r0 + tr * TM + a;
            acc[a][b] = (r < m && c < n) ? A[r + (size_t)c * ldda] : T(0);
        }
    }
    __syncthreads();
    for (int k = 0; k < ib; k++) {
        T l[TM], u[TN];
#pragma unroll
        for (int a = 0; a < TM; a++) l[a] = sL[k][tr * TM + a];
#pragma unroll
        for (int b = 0; b < TN; b++) u[b] = sU[k][tc * TN + b];
#pragma unroll
        for (int a = 0; a < TM; a++)
#pragma unroll
            for (int b = 0; b < TN; b++) acc[a][b] = Prec<T>::fma_(-l[a], u[b], acc[a][b]);
    }
#pragma unroll
    for (int b = 0; b < TN; b++) {
        const int c = c0 + tc * TN + b;
#pragma unroll
        for (int a = 0; a < TM; a++) {
            const int r = r0 + tr * TM + a;
            if (r < m && c < n) A[r + (size_t)c * ldda] = acc[a][b];
        }
    }
}

template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q)
{
    if (batch <= 0 || m == 0 || n == 0) return MAGMA_SUCCESS;
    cudaStream_t s = q->stream;
    const int mn = min(m, n);
    constexpr int BM = 64, BN = 64, TM = 4, TN = 4;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PANEL_SMEM_MAX + 1024);
        attr_set = true;
    }
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        T **dAb = dA + b0;
        int **ipb = ipiv + b0;
        int *infb = info + b0;
        for (int j0 = 0; j0 < mn; ) {
            const int pm = m - j0;
            int ib = min(PANEL_NB, mn - j0);
            while (ib > 1 && (size_t)pm * (ib + 1) * sizeof(T) + 2 * pm * sizeof(int) > PANEL_SMEM_MAX)
                ib /= 2;
            if ((size_t)pm * (ib + 1) * sizeof(T) + 2 * pm * sizeof(int) > PANEL_SMEM_MAX)
                return MAGMA_ERR_NOT_SUPPORTED;   // m too large for a shared-memory panel
            const size_t smem = (size_t)pm * (ib + 1) * sizeof(T) + 2 * (size_t)pm * sizeof(int);
            panel_kernel<T><<<nb, PANEL_THREADS, smem, s>>>(m, j0, ib, dAb, ldda, ipb, infb);
            const int ncl = (j0 + SWAP_W - 1) / SWAP_W;
            const int ncr = (n - j0 - ib + SWAP_W - 1) / SWAP_W;
            if (ncl + ncr > 0) {
                swap_trsm_kernel<T><<<dim3(ncl + ncr, nb), SWAP_THREADS, 0, s>>>(
                    m, n, j0, ib, dAb, ldda, ipb);
            }
            const int rm = m - j0 - ib, rn = n - j0 - ib;
            if (rm > 0 && rn > 0) {
                const int tiles_m = (rm + BM - 1) / BM, tiles_n = (rn + BN - 1) / BN;
                gemm_kernel<T, BM, BN, TM, TN><<<dim3(tiles_m * tiles_n, nb),
                                                 (BM / TM) * (BN / TN), 0, s>>>(
                    m, n, j0, ib, dAb, ldda, tiles_m);
            }
            j0 += ib;
        }
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Blocked solves.  One CTA per (matrix, group of SOLVE_NR right-hand sides);
// the right-hand sides live in shared memory.  Triangular blocks of 32 are
// solved by warp 0 with shuffles, the rows below/above are then updated by
// all threads; every element receives its updates in the oracle's order.

constexpr int SOLVE_THREADS = 256;
constexpr int SOLVE_NR = 8;

template <typename T, bool TRANS>
__global__ void __launch_bounds__(SOLVE_THREADS)
getrs_kernel(int n, int nrhs, T **dA_array, int ldda, int **ipiv_array, T **dB_array, int lddb)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sB = reinterpret_cast<T *>(smem_raw);   // [SOLVE_NR][n]
    const int tid = threadIdx.x;
    const int mat = blockIdx.y;
    const int c0 = blockIdx.x * SOLVE_NR;
    const int nr = min(SOLVE_NR, nrhs - c0);
    const T *A = dA_array[mat];
    const int *ipiv = ipiv_array[mat];
    T *B = dB_array[mat] + (size_t)c0 * lddb;

    for (int e = tid; e < SOLVE_NR * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        sB[c * n + i] = c < nr ? B[i + (size_t)c * lddb] : T(0);
    }
    __syncthreads();
    solve_smem<T, TRANS, SOLVE_NR>(n, A, ldda, ipiv, sB, nr);
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
    const size_t smem = (size_t)SOLVE_NR * n * sizeof(T);
    if (smem > 220 * 1024) return MAGMA_ERR_NOT_SUPPORTED;
    static bool attr_set[2] = {false, false};
    if (!attr_set[trans]) {
        if (trans)
            cudaFuncSetAttribute(getrs_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        else
            cudaFuncSetAttribute(getrs_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr_set[trans] = true;
    }
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        dim3 grid((nrhs + SOLVE_NR - 1) / SOLVE_NR, nb);
        if (trans)
            getrs_kernel<T, true><<<grid, SOLVE_THREADS, smem, q->stream>>>(n, nrhs, dA + b0, ldda, ipiv + b0, dB + b0, lddb);
        else
            getrs_kernel<T, false><<<grid, SOLVE_THREADS, smem, q->stream>>>(n, nrhs, dA + b0, ldda, ipiv + b0, dB + b0, lddb);
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

template magma_int_t blocked_getrf<double>(int, int, double **, int, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrf<float>(int, int, float **, int, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrs<double>(bool, int, int, double **, int, int **, double **, int, int, magma_queue_t);
template magma_int_t blocked_getrs<float>(bool, int, int, float **, int, int **, float **, int, int, magma_queue_t);

}  // namespace mlu
