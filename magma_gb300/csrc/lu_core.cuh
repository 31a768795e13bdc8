// lu_core.cuh -- the steps of one right-looking LU panel step as device
// functions, shared by the per-step kernels of the fixed-size path
// (lu_blocked.cu) and the persistent one-CTA-per-matrix kernel of the
// variable-size path (lu_vbatched.cu).  Both therefore perform the same
// floating-point operations in the same order as the CPU oracle.
//
// Restates, in one place: the fused panel (magmablas/zgetf2_kernels.cu:833-1058,
// magmablas/zgetf2_devicefunc.cuh:218-294), the pivot bookkeeping
// (magmablas/getrf_setup_pivinfo.cu:59-309), the row swaps
// (magmablas/zlaswp_device.cuh:25-84), the TRSM of U12
// (magmablas/ztrsm_batched_core.cpp) and the trailing update (cuBLAS dgemm in
// the reference, magmablas/zgemm_batched.cpp:60-89).
#pragma once
#include "common.cuh"

namespace mlu {

constexpr int PANEL_NB = 32;          // largest panel width
constexpr size_t PANEL_SMEM_MAX = 200 * 1024;   // shared memory for one panel
constexpr int SWAP_W = 32;            // columns per gather/scatter chunk
constexpr int GEMM_LDU = PANEL_NB + 4; // row stride of the transposed U12 tile in gemm_tile

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

// Two-level blocking of the FP32 factorisation: columns are factored in
// blocks of OUTER_NB (four 32-column panels); inside a block the steps update
// only the block's own columns, and the columns right of the block receive one
// rank-OUTER_NB update per block (lu_outer.cu).  For a matrix with mn =
// min(m, n), the block that starts at column bj ends at column
// bj + min(OUTER_NB, mn - bj); bj < 0 means no outer blocking (the steps
// update every column right of the panel).
constexpr int OUTER_NB = 128;
__host__ __device__ __forceinline__ int block_col_end(int bj, int m, int n)
{
    return bj < 0 ? n : min(n, bj + min(OUTER_NB, min(m, n) - bj));
}

// ---------------------------------------------------------------------------
// NOPIV (both panels): the pivot of column k is the diagonal entry, as in
// MAGMA's getrf_nopiv; a zero diagonal sets info and leaves the column
// unscaled, the same rule as a zero pivot column with pivoting.
//
// Panel factorisation of the pm x ib block at A (leading dimension lda) in
// shared memory.  `smem` must hold pm*(ib+1) T plus 2*pm ints.  Every thread
// of the block calls it.  On return the panel is written back in pivoted
// order, s_ipiv[k] holds the pivot position (relative to the panel's first
// row) chosen at column k, and the return value (valid in thread 0) is the
// 1-based column of the first zero pivot plus `col0`, or 0.
//
// Rows stay where they were loaded; sPos[i] is row i's position in LAPACK's
// current order and sRowAt the inverse.  Per column: per-thread then per-warp
// arg-max of |a| (63-bit integer keys, ties to the smaller position, idamax's
// NaN rule), one warp combines the warp winners and updates the maps, then
// every thread scales and updates only its own rows -- two barriers per
// column.
template <typename T, bool NOPIV = false>
__device__ __forceinline__ int panel_factor(int pm, int ib, T *A, int lda, unsigned char *smem, int *s_ipiv,
                            int col0)
{
    __shared__ unsigned s_whi[32], s_wlo[32], s_wpos[32];
    __shared__ int s_prow;
    __shared__ T s_piv, s_rcp;
    const int LDS = ib + 1;
    T *sP = reinterpret_cast<T *>(smem);
    int *sPos = reinterpret_cast<int *>(sP + (size_t)pm * LDS);
    int *sRowAt = sPos + pm;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthr = blockDim.x, nwarps = nthr >> 5;

    for (int j = 0; j < ib; j++)
        for (int i = tid; i < pm; i += nthr) sP[i * LDS + j] = A[i + (size_t)j * lda];
    for (int i = tid; i < pm; i += nthr) { sPos[i] = i; sRowAt[i] = i; }
    int info_local = 0;
    __syncthreads();

    for (int k = 0; k < ib; k++) {
        unsigned long long best = 0ull;
        unsigned bpos = 0xffffffffu;
        for (int i = tid; i < pm; i += nthr) {
            const int p = sPos[i];
            if (p >= k) {
                const T v = sP[i * LDS + k];
                unsigned long long mag = Prec<T>::absbits(v);
                if (Prec<T>::isnan_(v)) mag = (p == k) ? 0x7fffffffffffffffull : 0ull;
                if (NOPIV) mag = (p == k) ? 0x7fffffffffffffffull : 0ull;   // the diagonal
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
                if (!Prec<T>::nonzero(piv) && info_local == 0) info_local = col0 + k + 1;
            }
        }
        __syncthreads();
        const int prow = s_prow;
        const T piv = s_piv, r = s_rcp;
        const bool nz = Prec<T>::nonzero(piv);
        for (int i = tid; i < pm; i += nthr) {
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
    for (int j = 0; j < ib; j++)
        for (int i = tid; i < pm; i += nthr) A[sPos[i] + (size_t)j * lda] = sP[i * LDS + j];
    __syncthreads();
    return info_local;
}

// ---------------------------------------------------------------------------
// Register-resident panel factorisation, same arithmetic as panel_factor.
// 256 threads; thread t owns rows t + 256 r (r < RPT, pm <= 256 RPT).  The
// column loop is a real loop (an unrolled one is tens of kilobytes of
// straight-line code that each SM runs only a few times, and stalls on
// instruction fetch), so registers cannot be indexed by the column.  Instead
// a[r][0..] holds columns k..ib-1 of the row at step k: the update of step k
// writes column j into a[r][j-1], shifting the row by one column per step
// with no moves, and a[r][0] is always the current column.  A column leaving
// the registers is final (an L multiplier, or an entry of the U row of a
// pivot row, which leaves whole when it is chosen) and is stored to sP
// (shared, ib x panel_regs_ld columns, physical row order).  One barrier per
// column: each warp publishes its best candidate (key, position, remaining
// row) into a double-buffered table that every warp then reduces with
// shuffles.  Rows are written back to A in pivoted order, coalesced.
// Returns the first zero pivot column + col0 (1-based) or 0, valid in thread
// 0; s_ipiv[k] = position (0-based, panel-relative) chosen at step k.
constexpr int PANEL_REGS_THREADS = 256;

// NT: the CTA's threads (RPT * NT >= panel rows); 256 unless a shorter panel
// runs in a smaller CTA.
template <typename T, int RPT, int NT = PANEL_REGS_THREADS>
__host__ __device__ constexpr int panel_regs_ld() { return NT * RPT; }

// shared memory that panel_factor_regs<T, RPT, NOPIV, NT> needs from its caller
template <typename T, int RPT, int NT = PANEL_REGS_THREADS>
__host__ __device__ constexpr size_t panel_regs_smem_bytes()
{
    return (size_t)PANEL_NB * panel_regs_ld<T, RPT, NT>() * sizeof(T) +
           (size_t)panel_regs_ld<T, RPT, NT>() * sizeof(int);
}

template <typename T, int RPT, bool NOPIV = false, int NT = PANEL_REGS_THREADS>
__device__ __forceinline__ int panel_factor_regs(int pm, int ib, T *A, int lda, int *s_ipiv,
                                                 int col0, unsigned char *smem)
{
    constexpr int NW = NT / 32;
    constexpr int LDP = panel_regs_ld<T, RPT, NT>();
    __shared__ unsigned s_hi[2][NW], s_lo[2][NW], s_pos[2][NW];
    __shared__ __align__(16) T s_row[2][NW][PANEL_NB];
    T *sP = reinterpret_cast<T *>(smem);
    int *s_slot = reinterpret_cast<int *>(smem + (size_t)PANEL_NB * LDP * sizeof(T));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    T a[RPT][PANEL_NB];
    int pos[RPT];
    bool live[RPT];
#pragma unroll
    for (int r = 0; r < RPT; r++) {
        const int i = tid + r * NT;
        live[r] = i < pm;
        pos[r] = i;
#pragma unroll
        for (int j = 0; j < PANEL_NB; j++)
            a[r][j] = (i < pm && j < ib) ? A[i + (size_t)j * lda] : T(0);
    }
    int info_local = 0;

#pragma unroll 1
    for (int k = 0; k < ib; k++) {
        const int buf = k & 1;
        // best live row of this thread: largest key, ties to the smaller position
        unsigned long long best = 0ull;
        unsigned bpos = 0xffffffffu;
        int bslot = 0;
#pragma unroll
        for (int r = 0; r < RPT; r++) {
            if (live[r]) {
                const T v = a[r][0];
                unsigned long long mag = Prec<T>::absbits(v);
                if (Prec<T>::isnan_(v)) mag = (pos[r] == k) ? 0x7fffffffffffffffull : 0ull;
                if (NOPIV) mag = (pos[r] == k) ? 0x7fffffffffffffffull : 0ull;   // the diagonal
                const unsigned long long key = mag | 0x8000000000000000ull;
                if (key > best || (key == best && (unsigned)pos[r] < bpos)) {
                    best = key; bpos = pos[r]; bslot = r;
                }
            }
        }
        {
            const unsigned hi = (unsigned)(best >> 32), lo = (unsigned)best;
            const unsigned mhi = __reduce_max_sync(FULL, hi);
            const unsigned mlo = __reduce_max_sync(FULL, hi == mhi ? lo : 0u);
            const bool cand = hi == mhi && lo == mlo;
            const unsigned wpos = __reduce_min_sync(FULL, cand ? bpos : 0xffffffffu);
            if (lane == 0) { s_hi[buf][warp] = mhi; s_lo[buf][warp] = mlo; s_pos[buf][warp] = wpos; }
            if (cand && bpos == wpos && mhi != 0u) {
#pragma unroll
                for (int j = 0; j < PANEL_NB; j++) {
                    T v = a[0][j];
#pragma unroll
                    for (int r = 1; r < RPT; r++) v = (bslot == r) ? a[r][j] : v;
                    s_row[buf][warp][j] = v;
                }
            }
        }
        __syncthreads();
        // every warp reduces the NW warp winners with shuffles
        unsigned gpos, gw;
        {
            const unsigned h = lane < NW ? s_hi[buf][lane] : 0u;
            const unsigned l = lane < NW ? s_lo[buf][lane] : 0u;
            const unsigned p = lane < NW ? s_pos[buf][lane] : 0xffffffffu;
            const unsigned mh = __reduce_max_sync(FULL, h);
            const unsigned ml = __reduce_max_sync(FULL, h == mh ? l : 0u);
            const bool c = lane < NW && h == mh && l == ml;
            gpos = __reduce_min_sync(FULL, c ? p : 0xffffffffu);
            gw = __ffs(__ballot_sync(FULL, c && p == gpos)) - 1;
        }
        const T *prow = s_row[buf][gw];
        const T piv = prow[0];
        const bool nz = Prec<T>::nonzero(piv);
        // the reciprocal only in warps that still hold rows: on this part an FP64
        // division costs the same issue slots in a warp whose lanes do not need it
        bool any_live = false;
#pragma unroll
        for (int r = 0; r < RPT; r++) any_live |= live[r];
        T rcp = T(0);
        if (__any_sync(FULL, any_live)) rcp = T(1) / piv;
        if (tid == 0) {
            s_ipiv[k] = (int)gpos;
            if (!nz && info_local == 0) info_local = col0 + k + 1;
        }
#pragma unroll
        for (int r = 0; r < RPT; r++) {
            if (!live[r]) continue;
            const int slot = tid + r * NT;
            // interchange of positions k and gpos
            if (pos[r] == (int)gpos) pos[r] = k;
            else if (pos[r] == k) pos[r] = (int)gpos;
            if (pos[r] == k) {
                // the pivot row: its remaining entries are U(k, k..ib-1)
#pragma unroll
                for (int j = 0; j < PANEL_NB; j++)
                    if (j < ib - k) sP[(size_t)(k + j) * LDP + slot] = a[r][j];
                live[r] = false;
            } else {
                const T l = nz ? rscale(a[r][0], piv, rcp) : a[r][0];
                sP[(size_t)k * LDP + slot] = l;
                // the row's remaining columns are j < ib - k: groups of eight past
                // them are skipped (the same test in every lane of the block)
#pragma unroll
                for (int c = 0; c < PANEL_NB / 8; c++) {
                    if (8 * c + 1 < ib - k) {
#pragma unroll
                        for (int jj = 0; jj < 8; jj++) {
                            const int j = 8 * c + 1 + jj;
                            if (j < PANEL_NB) a[r][j - 1] = Prec<T>::fma_(-l, prow[j], a[r][j]);
                        }
                    }
                }
            }
        }
    }
    // write back in pivoted order: position -> slot map, then coalesced rows
#pragma unroll
    for (int r = 0; r < RPT; r++) {
        const int slot = tid + r * NT;
        if (slot < pm) s_slot[pos[r]] = slot;
    }
    __syncthreads();
    for (int j = 0; j < ib; j++) {
#pragma unroll
        for (int r = 0; r < RPT; r++) {
            const int p = tid + r * NT;
            if (p < pm) A[p + (size_t)j * lda] = sP[(size_t)j * LDP + s_slot[p]];
        }
    }
    __syncthreads();
    return info_local;
}

// ---------------------------------------------------------------------------
// Compound permutation of the sequential interchanges k = j0..j0+ib-1 with
// targets ipiv[k]-1 (1-based ipiv).  Built by warp 0 (threads 0..31 must call
// it) with ballots over a 64-entry table: s_row[e] is a touched row, s_src[e]
// the row whose original content ends up there.  The caller synchronises
// before using the table.
__device__ __forceinline__ void build_permutation(const int *ipiv, int j0, int ib, int *s_row, int *s_src,
                                         int *s_cnt)
{
    const int lane = threadIdx.x & 31;
    // all ib targets in one coalesced load, then broadcast by shuffles
    const int my_target = lane < ib ? ipiv[j0 + lane] - 1 : 0;
    int cnt = 0;
    int r0 = -1, r1 = -1, s0 = -1, s1 = -1;   // this lane's entries lane and lane+32
    for (int k = 0; k < ib; k++) {
        const int a = j0 + k, b = __shfl_sync(FULL, my_target, k);
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
        const int va = __shfl_sync(FULL, ia < 32 ? s0 : s1, ia & 31);
        const int vb = __shfl_sync(FULL, ibb < 32 ? s0 : s1, ibb & 31);
        if (lane == (ia & 31)) { if (ia < 32) s0 = vb; else s1 = vb; }
        if (lane == (ibb & 31)) { if (ibb < 32) s0 = va; else s1 = va; }
    }
    s_row[lane] = r0; s_src[lane] = s0;
    s_row[lane + 32] = r1; s_src[lane + 32] = s1;
    if (lane == 0) *s_cnt = cnt;
}

// Moves the touched rows of columns [c0, c1) of A (ld lda): gather all sources
// into s_tmp (2*PANEL_NB x (SWAP_W+1)), then scatter, SWAP_W columns at a time.
// All threads call it; it synchronises internally.
template <typename T>
__device__ __forceinline__ void apply_permutation(T *A, int lda, int c0, int c1, const int *s_row, const int *s_src,
                                  int cnt, T *s_tmp)
{
    // rows run fastest across threads, so runs of adjacent rows coalesce;
    // eight loads per thread in flight before their stores
    const int tid = threadIdx.x, nthr = blockDim.x;
    if (cnt == 0) return;
    for (int cb = c0; cb < c1; cb += SWAP_W) {
        const int w = min(SWAP_W, c1 - cb);
        const int total = cnt * w;
        for (int e0 = tid; e0 < total; e0 += 8 * nthr) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * nthr;
                if (e < total) v[u] = A[s_src[e % cnt] + (size_t)(cb + e / cnt) * lda];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * nthr;
                if (e < total) s_tmp[(e % cnt) * (SWAP_W + 1) + e / cnt] = v[u];
            }
        }
        __syncthreads();
        for (int e = tid; e < cnt * w; e += nthr) {
            const int pr = e % cnt, c = e / cnt;
            A[s_row[pr] + (size_t)(cb + c) * lda] = s_tmp[pr * (SWAP_W + 1) + c];
        }
        __syncthreads();
    }
}

// U12 = L11^{-1} A12 for the columns [c0, c1) of the ib rows starting at row
// j0 (L11 unit lower, at (j0, j0)), the right-hand sides staged in shared
// memory (sbuf: PANEL_NB x chunk T): one thread per column, updates
// u_i = fma(-l_it, u_t, u_i) for t ascending.  All threads call it.
template <typename T>
__device__ __forceinline__ void trsm_l11_smem(T *A, int lda, int j0, int ib, int c0, int c1,
                                              T *sbuf, int chunk)
{
    __shared__ T s_L[PANEL_NB][PANEL_NB + 1];
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int e = tid; e < ib * ib; e += nthr) {
        const int i = e % ib, t = e / ib;
        s_L[i][t] = A[j0 + i + (size_t)(j0 + t) * lda];
    }
    for (int cb = c0; cb < c1; cb += chunk) {
        const int w = min(chunk, c1 - cb);
        __syncthreads();
        const int total = ib * w;
        for (int e0 = tid; e0 < total; e0 += 8 * nthr) {   // coalesced down each column
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * nthr;
                if (e < total) v[u] = A[j0 + e % ib + (size_t)(cb + e / ib) * lda];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * nthr;
                if (e < total) sbuf[(e % ib) * chunk + e / ib] = v[u];
            }
        }
        __syncthreads();
        for (int c = tid; c < w; c += nthr) {
            for (int t = 0; t < ib; t++) {
                const T ut = sbuf[t * chunk + c];
                for (int i = t + 1; i < ib; i++)
                    sbuf[i * chunk + c] = Prec<T>::fma_(-s_L[i][t], ut, sbuf[i * chunk + c]);
            }
        }
        __syncthreads();
        for (int e = tid; e < ib * w; e += nthr) {
            const int i = e % ib, c = e / ib;
            A[j0 + i + (size_t)(cb + c) * lda] = sbuf[i * chunk + c];
        }
    }
    __syncthreads();
}

// One BM x BN tile of A22 -= L21 * U12 with rows from r0 and columns from c0
// (rows >= m or columns >= n skipped).  L21 columns j0..j0+ib, U12 rows
// j0..j0+ib.  sL, sU: PANEL_NB x BM and BN x GEMM_LDU T.  Called by exactly
// (BM/TM)*(BN/TN) threads; synchronises on entry.  Every element is updated
// acc = fma(-l_k, u_k, acc) for k ascending.  The U12 tile is stored
// transposed (sU[j][k]) so that its store (lanes down a column of A) and the
// compute loop's reads (4 consecutive k per thread) are free of bank conflicts.
//
// SYRK (the Cholesky trailing update A22 -= L21 L21^T): U12 is L21^T, read
// from the rows c0.. of the panel columns, and only elements on or below the
// diagonal (row >= column) are stored.
template <typename T, int BM, int BN, int TM, int TN, bool SYRK = false>
__device__ __forceinline__ void gemm_tile(T *A, int lda, int m, int n, int j0, int ib, int r0, int c0, T *sL,
                          T *sU)
{
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int LU_LOADS = PANEL_NB * (BM > BN ? BM : BN) / NT;   // per thread, at most
    const int tid = threadIdx.x;
    __syncthreads();
    {
        // all of this thread's L21 and U12 loads in flight before the stores
        T vl[LU_LOADS], vu[LU_LOADS];
#pragma unroll
        for (int u = 0; u < LU_LOADS; u++) {
            const int e = tid + u * NT;
            const int i = e % BM, kl = e / BM;
            vl[u] = (kl < ib && r0 + i < m) ? A[r0 + i + (size_t)(j0 + kl) * lda] : T(0);
            const int ku = SYRK ? e / BN : e % ib, j = SYRK ? e % BN : e / ib;
            vu[u] = (e < ib * BN && c0 + j < n)
                        ? (SYRK ? A[c0 + j + (size_t)(j0 + ku) * lda] : A[j0 + ku + (size_t)(c0 + j) * lda])
                        : T(0);
        }
#pragma unroll
        for (int u = 0; u < LU_LOADS; u++) {
            const int e = tid + u * NT;
            if (e < ib * BM) sL[(e / BM) * BM + e % BM] = vl[u];
            const int ku = SYRK ? e / BN : e % ib, j = SYRK ? e % BN : e / ib;
            if (e < ib * BN) sU[j * GEMM_LDU + ku] = vu[u];
        }
    }
    const int tr = tid % (BM / TM), tc = tid / (BM / TM);
    T acc[TM][TN];
#pragma unroll
    for (int b = 0; b < TN; b++) {
        const int c = c0 + tc * TN + b;
#pragma unroll
        for (int a = 0; a < TM; a++) {
            const int r = r0 + tr * TM + a;
            acc[a][b] = (r < m && c < n) ? A[r + (size_t)c * lda] : T(0);
        }
    }
    __syncthreads();
    // Nothing of this thread's block is stored when its columns (or rows) lie past
    // the matrix, or (SYRK) the block lies above the diagonal: it leaves now (no
    // barrier follows).  A warp's lanes share their columns, so at the right edge of
    // the trailing matrix whole warps issue no FMAs, which on this part's FP64 pipe
    // cost their issue slots whether or not any lane keeps the result.
    if (c0 + tc * TN >= n || r0 + tr * TM >= m) return;
    if (SYRK && r0 + tr * TM + TM - 1 < c0 + tc * TN) return;
    int k = 0;
    // four k at a time: each thread's U entries for 4 consecutive k are contiguous
    for (; k + 4 <= ib; k += 4) {
        T u[TN][4];
#pragma unroll
        for (int b = 0; b < TN; b++)
#pragma unroll
            for (int kk = 0; kk < 4; kk++) u[b][kk] = sU[(tc * TN + b) * GEMM_LDU + k + kk];
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            T l[TM];
#pragma unroll
            for (int a = 0; a < TM; a++) l[a] = sL[(k + kk) * BM + tr * TM + a];
#pragma unroll
            for (int a = 0; a < TM; a++)
#pragma unroll
                for (int b = 0; b < TN; b++) acc[a][b] = Prec<T>::fma_(-l[a], u[b][kk], acc[a][b]);
        }
    }
    for (; k < ib; k++) {
        T l[TM], u[TN];
#pragma unroll
        for (int a = 0; a < TM; a++) l[a] = sL[k * BM + tr * TM + a];
#pragma unroll
        for (int b = 0; b < TN; b++) u[b] = sU[(tc * TN + b) * GEMM_LDU + k];
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
            if (r < m && c < n && (!SYRK || r >= c)) A[r + (size_t)c * lda] = acc[a][b];
        }
    }
}

// Panel width for a panel of pm rows whose shared-memory copy must fit in
// `budget` bytes: 32, halved until it fits (at least 1).
template <typename T>
__host__ __device__ inline int panel_width(int pm, int want, size_t budget)
{
    int ib = want;
    while (ib > 1 && (size_t)pm * (ib + 1) * sizeof(T) + 2 * (size_t)pm * sizeof(int) > budget)
        ib >>= 1;
    return ib;
}

template <typename T>
__host__ __device__ inline size_t panel_smem_bytes(int pm, int ib)
{
    return (size_t)pm * (ib + 1) * sizeof(T) + 2 * (size_t)pm * sizeof(int);
}

}  // namespace mlu
