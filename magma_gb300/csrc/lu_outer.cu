// lu_outer.cu -- the rank-128 update of the two-level blocked FP32 LU.
//
// MAGMA factors a batch in blocks of nb = 128 columns, each block by recursive
// panels of recnb = 32 (control/get_batched_crossover.cpp:300-305,
// src/zgetrf_batched.cpp:149-203, src/zgetrf_panel_batched.cpp:102-196), and
// gives each block's trailing matrix one row interchange pass
// (magmablas/zlaswp_batched.cu:48-89), one TRSM (magmablas/ztrsm_batched_core.cpp)
// and one rank-128 cublasSgemmBatched (magmablas/zgemm_batched.cpp:60-89).
// Here the four 32-column panels of a block and the updates inside the block
// are the step kernels of lu_blocked.cu, and one launch does the rest for all
// the columns right of the block:
//
//   outer_update_kernel  one CTA per (matrix, 128-column tile right of the block)
//     1. resolves the block's interchanges (up to 128): where each top row of
//        the block gets its new content from, and for each row below the block
//        that an interchange touches, which original top row it receives;
//     2. gathers the tile's interchanged top rows into shared memory and
//        solves U12 = L11^{-1} A12 there, 32 rows at a time (a triangular solve
//        by one thread per column, then a rank-32 update of the rows below);
//     3. sweeps the rows below the block in 128-row tiles: the A22 tile lives
//        in registers (8 x 8 elements per thread), L21 streams through shared
//        memory in 32-column stages (cp.async, double-buffered and continuous
//        across the tiles), and every element is updated acc = fma(-l, u, acc)
//        for k ascending;
//     4. writes U12 back last, so that a row below that receives an original
//        top row can still read it from its old place during the sweep.
//
// Before this launch, left_swaps_kernel (LEFT_IN_BLOCK) has applied the
// block's later interchanges to its earlier panels, so L11 and L21 are read in
// their final row order with 16-byte copies.  Per element these are the
// operations of the unblocked elimination in the same order, so the factors
// are bit-identical to the oracle's.
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace mlu {

constexpr int OB_TN = 128;                   // columns per CTA
constexpr int OB_TM = 128;                   // rows of A22 per sweep tile
constexpr int OB_KC = 32;                    // columns of L11 per diagonal block of the solve
constexpr int OB_SK = 32;                    // columns of L21 per sweep stage
constexpr int OB_RING = 2;                   // sweep stages in flight (ring)
constexpr int OB_THREADS = 256;
constexpr int OB_MAX_ROWS = 1024;            // rows per matrix (register panels, deferred interchanges)
constexpr int OB_U_FLOATS = OUTER_NB * OB_TN;
constexpr int OB_STAGE_FLOATS = OB_KC * OB_TM;     // one L11 stage of the solve (two of them)
constexpr int OB_SSTAGE_FLOATS = OB_SK * OB_TM;    // one L21 stage of the sweep (four of them)
constexpr size_t OB_SMEM = sizeof(float) * (OB_U_FLOATS + 2 * OB_STAGE_FLOATS);   // 96 KB
static_assert(OB_TM == 128 && OB_TN == 128 && OB_THREADS == 256, "8 x 8 elements per thread");
static_assert(OB_RING * OB_SSTAGE_FLOATS <= 2 * OB_STAGE_FLOATS, "the ring reuses the solve's stages");
static_assert(OUTER_NB % OB_SK == 0 && OB_SK % 8 == 0, "sweep stages");

// Index of U12 element (k, c) in shared memory.  Groups of four columns (16
// bytes) are permuted by k mod 8, so that eight consecutive k of four columns
// (the gather) and one row read four columns per thread (the update) are both
// free of bank conflicts.
__device__ __forceinline__ int ob_uidx(int k, int c)
{
    return k * OB_TN + ((((c >> 2) ^ (k & 7))) << 2) + (c & 3);
}

// Row x followed through the block's interchanges k = K-1 .. 0 (k relative to
// the block's first column J, targets s_piv, 0-based global rows): as a
// gather, row x of the interchanged order holds the row returned here.
__device__ __forceinline__ int ob_resolve(int x, int J, int K, const int *s_piv)
{
    int v = x;
    for (int k = K - 1; k >= 0; k--) {
        const int a = J + k, b = s_piv[k];
        v = v == a ? b : (v == b ? a : v);
    }
    return v;
}

// 64 updates of one k: rows la (4) and lb (4) of L against columns ua (4) and
// ub (4) of U, acc[h][i][g][j] for row h*64 + tr*4 + i and column g*64 + tc*4 + j.
// Column-major order (one U value against the eight L values) and a two-step
// unroll of the k loop keep the kernel within 128 registers without spilling
// (measured: 1.43 against 1.50 ms per factorisation with row-major order and
// an eight-step unroll, which spilled).
__device__ __forceinline__ void ob_fma(float (&acc)[2][4][2][4], const float4 &la, const float4 &lb,
                                       const float4 &ua, const float4 &ub)
{
    const float l[2][4] = {{la.x, la.y, la.z, la.w}, {lb.x, lb.y, lb.z, lb.w}};
    const float u[2][4] = {{ua.x, ua.y, ua.z, ua.w}, {ub.x, ub.y, ub.z, ub.w}};
#pragma unroll
    for (int g = 0; g < 2; g++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int i = 0; i < 4; i++) acc[h][i][g][j] = fmaf(-l[h][i], u[g][j], acc[h][i][g][j]);
}

// Triangular solve of the 32-row diagonal block kb for column c (one thread
// per column): x_i = fma(-l_it, x_t, x_i) for t < i ascending, rows from kt on
// (the block's last rows when K is not a multiple of 32) untouched.
template <bool FULLB>
__device__ __forceinline__ void ob_diag_solve(float *sU, const float *Lp, int kb, int kt, int c)
{
    float x[OB_KC];
#pragma unroll
    for (int r = 0; r < OB_KC; r++) x[r] = (FULLB || r < kt) ? sU[ob_uidx(OB_KC * kb + r, c)] : 0.f;
#pragma unroll
    for (int t = 0; t < OB_KC - 1; t++) {
        if (FULLB || t < kt) {
            const float xt = x[t];
            const float *lt = Lp + t * OUTER_NB + OB_KC * kb;   // L(32kb + r, 32kb + t), r = 0..31
#pragma unroll
            for (int r = t + 1; r < OB_KC; r++)
                if (FULLB || r < kt) x[r] = fmaf(-lt[r], xt, x[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < OB_KC; r++)
        if (FULLB || r < kt) sU[ob_uidx(OB_KC * kb + r, c)] = x[r];
}

// Rows [r0, r0 + 128) x SK columns from column col of A (leading dimension ld)
// into dst[t][i] (t < kt columns, i < 128 rows; rows >= m and columns >= kt
// read as zero), by cp.async: 16-byte copies of four rows when `vec`.
template <int SK = OB_KC>
__device__ __forceinline__ void ob_stage(float *dst, const float *A, size_t ld, int r0, int m, int col,
                                         int kt, bool vec, int tid)
{
    if (vec) {
#pragma unroll
        for (int u = 0; u < SK * OB_TM / 4 / OB_THREADS; u++) {
            const int e = tid + u * OB_THREADS, i4 = (e % (OB_TM / 4)) * 4, t = e / (OB_TM / 4);
            const int r = r0 + i4;
            const float *src = A + r + (size_t)(col + t) * ld;
            const unsigned d = (unsigned)__cvta_generic_to_shared(dst + t * OB_TM + i4);
            if (t < kt && r + 3 < m) {
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++)
                    cp_async_elem<4>(dst + t * OB_TM + i4 + q, t < kt && r + q < m ? src + q : A,
                                     t < kt && r + q < m);
            }
        }
    } else {
#pragma unroll 4
        for (int u = 0; u < SK * OB_TM / OB_THREADS; u++) {
            const int e = tid + u * OB_THREADS, i = e % OB_TM, t = e / OB_TM;
            const bool valid = r0 + i < m && t < kt;
            cp_async_elem<4>(dst + t * OB_TM + i, valid ? A + r0 + i + (size_t)(col + t) * ld : A, valid);
        }
    }
    cp_async_commit();
}

template <typename H> __device__ __forceinline__ H ob_to_half(float x);
template <> __device__ __forceinline__ float ob_to_half<float>(float x) { return x; }
template <> __device__ __forceinline__ __nv_bfloat16 ob_to_half<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <> __device__ __forceinline__ __half ob_to_half<__half>(float x) { return __float2half_rn(x); }

// TC = false: the whole update on the FP32 pipes (steps 1-4 above).
// TC = true (the tensor-core forms, lu_tc.cu): steps 1-3 and 5 only, plus
// what the tensor-core update needs to run in place afterwards -- the rows
// below the block that receive an original top row get it now, and U12 is
// rounded to H into the staging rows Ub[mat][column - E][0..128) (K-major,
// zero for k >= K), upad rows per matrix.
template <bool TC, typename H>
__global__ void __launch_bounds__(OB_THREADS, 2)
outer_update_kernel(int m, int n, int J, float **dA_array, int ldda, int **ipiv_array, StepSizes vs,
                    H *Ub, int upad)
{
    extern __shared__ __align__(16) float ob_smem[];
    float *sU = ob_smem;                          // [OUTER_NB][OB_TN], swizzled (ob_uidx)
    float *sL = ob_smem + OB_U_FLOATS;            // [2][OB_KC][OB_TM]: L11 / L21 chunks, k-major
    __shared__ int s_piv[OUTER_NB];               // the block's interchange targets
    __shared__ int s_top[OUTER_NB];               // new top row i comes from row s_top[i]
    __shared__ unsigned s_dmask[OB_MAX_ROWS / 32];   // rows below the block that receive a top row
    __shared__ int s_dsrc[OUTER_NB];                 // ... and which (listed per interchange)
    __shared__ unsigned char s_didx[OB_MAX_ROWS];    // row - E -> index into s_dsrc
    __shared__ int s_drow[TC ? OUTER_NB : 1];        // (TC) the row of entry e, row - E
    __shared__ int s_nt;
    const int mat = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int K = OUTER_NB;
    if (!vs.get(mat, J, m, n, ldda, K)) return;   // K: the block's width for this matrix
    const int E = J + K;                          // first column (and row) after the block
    const int c0 = E + blockIdx.x * OB_TN;
    if (c0 >= n) return;
    const int w = min(OB_TN, n - c0);
    float *A = dA_array[mat];
    const size_t ld = ldda;
    // 16-byte copies and vector accesses of four rows need aligned columns and rows
    const bool vec = (ld & 3) == 0 && ((uintptr_t)A & 15) == 0 && (J & 3) == 0 && (K & 3) == 0;

    // 1. interchanges: threads 0..127 follow the block's top rows, threads
    //    128..255 the pivot rows below the block.  A row below the block that an
    //    interchange touches always ends up holding an original top row.
    if (tid < OUTER_NB)
        s_piv[tid] = tid < K ? (ipiv_array ? ipiv_array[mat][J + tid] - 1 : J + tid) : 0;
    if (tid < K && !MLU_BC2(s_piv[tid], 0, m, 1, 101)) s_piv[tid] = J + tid;
    if (tid < OB_MAX_ROWS / 32) s_dmask[tid] = 0u;
    if (tid == 0) s_nt = 0;
    __syncthreads();
    if (tid < OUTER_NB) {
        if (tid < K) s_top[tid] = ob_resolve(J + tid, J, K, s_piv);
    } else {
        const int k = tid - OUTER_NB;
        if (k < K && s_piv[k] >= E) {
            // listed once per interchange that names the row (duplicates agree)
            const int e = atomicAdd(&s_nt, 1);
            const int row = s_piv[k] - E;
            s_dsrc[e] = ob_resolve(s_piv[k], J, K, s_piv);
            s_didx[row] = (unsigned char)e;
            if (TC) s_drow[TC ? e : 0] = row;
            atomicOr(&s_dmask[row >> 5], 1u << (row & 31));
        }
    }
    __syncthreads();

    // 2. the tile's interchanged top rows: sU[k][c] = A(s_top[k], c0 + c); a warp
    //    reads eight consecutive k of four columns, 32 loads in flight per thread
    for (int u0 = 0; u0 < OB_U_FLOATS / OB_THREADS; u0 += 32) {
        float v[32];
#pragma unroll
        for (int u = 0; u < 32; u++) {
            const int idx = tid + (u0 + u) * OB_THREADS;
            const int k = ((idx >> 5) & 15) * 8 + (idx & 7), c = (idx >> 9) * 4 + ((idx >> 3) & 3);
            v[u] = (k < K && c < w && MLU_BC2(s_top[k], c0 + c, m, n, 102)) ? A[s_top[k] + (size_t)(c0 + c) * ld]
                                                                           : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 32; u++) {
            const int idx = tid + (u0 + u) * OB_THREADS;
            const int k = ((idx >> 5) & 15) * 8 + (idx & 7), c = (idx >> 9) * 4 + ((idx >> 3) & 3);
            sU[ob_uidx(k, c)] = v[u];
        }
    }

    // micro-tile of this thread: rows h*64 + tr*4 + i, columns g*64 + tc*4 + j;
    // a warp covers 32 consecutive rows of each half and 16 columns of each half
    const int tr = ((warp & 1) << 3) | (lane & 7);
    const int tc = ((warp >> 1) << 2) | (lane >> 3);
    const int nkb = (K + OB_KC - 1) / OB_KC;

    // 3. U12 = L11^{-1} A12, 32 rows at a time; stage kb holds L11's column panel
    //    kb (rows J.. of columns J + 32kb ..), in final row order (the block's
    //    interchanges were applied to its columns after its last panel)
    ob_stage(sL, A, ld, J, E, J, min(OB_KC, K), vec, tid);
    for (int kb = 0; kb < nkb; kb++) {
        if (kb + 1 < nkb) {
            ob_stage(sL + ((kb + 1) & 1) * OB_STAGE_FLOATS, A, ld, J, E, J + OB_KC * (kb + 1),
                     min(OB_KC, K - OB_KC * (kb + 1)), vec, tid);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const float *Lp = sL + (kb & 1) * OB_STAGE_FLOATS;
        const int kt = min(OB_KC, K - OB_KC * kb);
        if (tid < w) {
            if (kt == OB_KC) ob_diag_solve<true>(sU, Lp, kb, kt, tid);
            else ob_diag_solve<false>(sU, Lp, kb, kt, tid);
        }
        __syncthreads();
        if (OB_KC * (kb + 1) < K) {
            // rows 32(kb+1).. of the block: rank-kt update with the rows just solved;
            // a warp's 32 rows of a half are all below the diagonal block or none are
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (h * 64 + (warp & 1) * 32 < OB_KC * (kb + 1)) continue;
                float acc[4][2][4];
                const int rb = h * 64 + tr * 4;
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int g = 0; g < 2; g++)
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[i][g][j] = sU[ob_uidx(rb + i, g * 64 + tc * 4 + j)];
#pragma unroll 4
                for (int t = 0; t < kt; t++) {
                    const int k = OB_KC * kb + t;
                    const float4 l4 = *reinterpret_cast<const float4 *>(Lp + t * OUTER_NB + rb);
                    const float4 ua = *reinterpret_cast<const float4 *>(sU + k * OB_TN + ((tc ^ (k & 7)) << 2));
                    const float4 ub =
                        *reinterpret_cast<const float4 *>(sU + k * OB_TN + (((16 + tc) ^ (k & 7)) << 2));
                    const float l[4] = {l4.x, l4.y, l4.z, l4.w};
                    const float u[2][4] = {{ua.x, ua.y, ua.z, ua.w}, {ub.x, ub.y, ub.z, ub.w}};
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int g = 0; g < 2; g++)
#pragma unroll
                            for (int j = 0; j < 4; j++) acc[i][g][j] = fmaf(-l[i], u[g][j], acc[i][g][j]);
                }
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int g = 0; g < 2; g++)
#pragma unroll
                        for (int j = 0; j < 4; j++) sU[ob_uidx(rb + i, g * 64 + tc * 4 + j)] = acc[i][g][j];
            }
        }
        __syncthreads();
    }

    // 4. A22 -= L21 U12, 128 rows at a time.  L21 streams through a ring of
    //    OB_RING stages of OB_SK columns, continuous across the row tiles: stage
    //    g holds columns J + OB_SK (g mod nsk) of tile g / nsk and is issued
    //    OB_RING - 1 stages ahead; one barrier per stage.
    const int below = TC ? 0 : m - E;             // TC: the tensor cores update A22
    const int ntiles = below > 0 ? (below + OB_TM - 1) / OB_TM : 0;
    const int nsk = (K + OB_SK - 1) / OB_SK;       // stages per tile
    const int nst = ntiles * nsk;
    auto stage_l21 = [&](int g) {
        if (g < nst) {
            const int q = g / nsk, kc = g % nsk;
            ob_stage<OB_SK>(sL + (g % OB_RING) * OB_SSTAGE_FLOATS, A, ld, E + q * OB_TM, m, J + OB_SK * kc,
                            min(OB_SK, K - OB_SK * kc), vec, tid);
        } else {
            cp_async_commit();                    // empty group: keeps the group count uniform
        }
    };
#pragma unroll
    for (int g = 0; g < OB_RING - 1; g++) stage_l21(g);
    float acc[2][4][2][4];
    for (int g = 0; g < nst; g++) {
        const int q = g / nsk, kc = g % nsk;
        const int r0 = E + q * OB_TM;
        if (kc == 0) {
            // the tile into registers; a row that receives an original top row reads it there
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int rb = h * 64 + tr * 4;
                const int rel = r0 - E + rb;           // row index below the block
                const unsigned dm = rel < OB_MAX_ROWS ? (s_dmask[rel >> 5] >> (rel & 31)) & 0xfu : 0u;
                const bool v4 = vec && r0 + rb + 3 < m;
#pragma unroll
                for (int gg = 0; gg < 2; gg++)
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int col = gg * 64 + tc * 4 + j;
                        const float *colp = A + (size_t)(c0 + col) * ld;
                        if (v4 && col < w && MLU_BC2(r0 + rb + 3, c0 + col, m, n, 103)) {
                            const float4 x = *reinterpret_cast<const float4 *>(colp + r0 + rb);
                            acc[h][0][gg][j] = x.x;
                            acc[h][1][gg][j] = x.y;
                            acc[h][2][gg][j] = x.z;
                            acc[h][3][gg][j] = x.w;
                        } else {
#pragma unroll
                            for (int i = 0; i < 4; i++)
                                acc[h][i][gg][j] =
                                    (r0 + rb + i < m && col < w && MLU_BC2(r0 + rb + i, c0 + col, m, n, 104))
                                        ? colp[r0 + rb + i] : 0.f;
                        }
                    }
                if (dm) {
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        if (dm & (1u << i)) {
                            const int src = s_dsrc[s_didx[rel + i]];
#pragma unroll
                            for (int gg = 0; gg < 2; gg++)
#pragma unroll
                                for (int j = 0; j < 4; j++) {
                                    const int col = gg * 64 + tc * 4 + j;
                                    if (col < w && MLU_BC2(src, c0 + col, m, n, 105))
                                        acc[h][i][gg][j] = A[src + (size_t)(c0 + col) * ld];
                                }
                        }
                    }
                }
            }
        }
        cp_async_wait<OB_RING - 2>();             // stage g has landed (younger ones may be in flight)
        __syncthreads();                          // ... for every thread; stage g-1 is free
        stage_l21(g + OB_RING - 1);
        const float *Lc = sL + (g % OB_RING) * OB_SSTAGE_FLOATS;
        const int kt = min(OB_SK, K - OB_SK * kc);
        if (kt == OB_SK) {
#pragma unroll 2
            for (int t = 0; t < OB_SK; t++) {
                const int k = OB_SK * kc + t;
                const float4 la = *reinterpret_cast<const float4 *>(Lc + t * OB_TM + tr * 4);
                const float4 lb = *reinterpret_cast<const float4 *>(Lc + t * OB_TM + 64 + tr * 4);
                const float4 ua = *reinterpret_cast<const float4 *>(sU + k * OB_TN + ((tc ^ (t & 7)) << 2));
                const float4 ub =
                    *reinterpret_cast<const float4 *>(sU + k * OB_TN + (((16 + tc) ^ (t & 7)) << 2));
                ob_fma(acc, la, lb, ua, ub);
            }
        } else {
            for (int t = 0; t < kt; t++) {
                const int k = OB_SK * kc + t;
                const float4 la = *reinterpret_cast<const float4 *>(Lc + t * OB_TM + tr * 4);
                const float4 lb = *reinterpret_cast<const float4 *>(Lc + t * OB_TM + 64 + tr * 4);
                const float4 ua = *reinterpret_cast<const float4 *>(sU + k * OB_TN + ((tc ^ (k & 7)) << 2));
                const float4 ub =
                    *reinterpret_cast<const float4 *>(sU + k * OB_TN + (((16 + tc) ^ (k & 7)) << 2));
                ob_fma(acc, la, lb, ua, ub);
            }
        }
        if (kc == nsk - 1) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int rb = h * 64 + tr * 4;
                const bool v4 = vec && r0 + rb + 3 < m;
#pragma unroll
                for (int gg = 0; gg < 2; gg++)
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int col = gg * 64 + tc * 4 + j;
                        if (col >= w) continue;
                        float *colp = A + (size_t)(c0 + col) * ld + r0 + rb;
                        if (v4 && MLU_BC2(r0 + rb + 3, c0 + col, m, n, 106)) {
                            *reinterpret_cast<float4 *>(colp) =
                                make_float4(acc[h][0][gg][j], acc[h][1][gg][j], acc[h][2][gg][j], acc[h][3][gg][j]);
                        } else {
#pragma unroll
                            for (int i = 0; i < 4; i++)
                                if (r0 + rb + i < m && MLU_BC2(r0 + rb + i, c0 + col, m, n, 107))
                                    colp[i] = acc[h][i][gg][j];
                        }
                    }
            }
        }
    }
    cp_async_wait<0>();

    if constexpr (TC) {
        // rows below that receive an original top row take it now (the top rows
        // are still original); then U12 rounded to H for the tensor cores
        const int nt = s_nt;
        for (int x = tid; x < nt * w; x += OB_THREADS) {
            const int e = x % nt, c = x / nt;
            float *colp = A + (size_t)(c0 + c) * ld;
            if (MLU_BC2(E + s_drow[e], c0 + c, m, n, 108) && MLU_BC2(s_dsrc[e], c0 + c, m, n, 109))
                colp[E + s_drow[e]] = colp[s_dsrc[e]];
        }
        H *U = Ub + (size_t)mat * upad * OUTER_NB + (size_t)(c0 - E) * OUTER_NB;
#pragma unroll 4
        for (int u = 0; u < OB_U_FLOATS / OB_THREADS; u++) {
            const int idx = tid + u * OB_THREADS, k = idx & (OUTER_NB - 1), c = idx / OUTER_NB;
            if (c < w) U[(size_t)c * OUTER_NB + k] = ob_to_half<H>(k < K ? sU[ob_uidx(k, c)] : 0.f);
        }
        __syncthreads();                          // the copies read top rows that step 5 rewrites
    }

    // 5. U12 into the block's top rows of the tile (read by no other CTA)
#pragma unroll 4
    for (int u = 0; u < OB_U_FLOATS / OB_THREADS; u++) {
        const int idx = tid + u * OB_THREADS;
        const int k = ((idx >> 5) & 15) * 8 + (idx & 7), c = (idx >> 9) * 4 + ((idx >> 3) & 3);
        if (k < K && c < w && MLU_BC2(J + k, c0 + c, m, n, 110)) A[J + k + (size_t)(c0 + c) * ld] = sU[ob_uidx(k, c)];
    }
}

// The rank-K update right of the block that starts at column J, for every
// matrix of the batch (m, n: the uniform sizes, or the maxima of a
// variable-size batch whose sizes are in vs).
magma_int_t outer_update(int m, int n, int J, float **dA, int ldda, int **ipiv, StepSizes vs,
                         int batch, magma_queue_t q)
{
    static size_t dyn[MLU_MAX_DEVICES];
    if (mlu_device_cached(dyn, [] { return mlu_allow_dynamic_smem(outer_update_kernel<false, float>); }) <
        OB_SMEM)
        return MAGMA_ERR_NOT_SUPPORTED;
    const int K = min(OUTER_NB, min(m, n) - J);
    // a variable-size batch: a matrix whose block is narrower starts its tiles earlier
    const int first = vs.m_arr ? J + 1 : J + K;
    if (K <= 0 || first >= n) return MAGMA_SUCCESS;
    const int tiles = (n - first + OB_TN - 1) / OB_TN;
    cudaStream_t s = q->stream;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        StepSizes v = vs;
        if (v.m_arr) {
            v.m_arr += b0;
            v.n_arr += b0;
            v.ld_arr += b0;
        }
        MLU_LAUNCH(mlu::KC_OUTER, s, outer_update_kernel<false, float><<<dim3(tiles, nb), OB_THREADS, OB_SMEM, s>>>(
            m, n, J, dA + b0, ldda, ipiv ? ipiv + b0 : nullptr, v, nullptr, 0));
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

// Steps 1-3 of the update right of block J for the tensor-core forms, uniform
// batch of m x n matrices: the interchanges (rows below applied in place), U12
// in place, and U12 rounded to H into Ub ([batch][upad][128]).
template <typename H>
magma_int_t outer_prep_tc(int m, int n, int J, float **dA, int ldda, int **ipiv, int batch, H *Ub,
                          int upad, magma_queue_t q)
{
    static size_t dyn[MLU_MAX_DEVICES];
    if (mlu_device_cached(dyn, [] { return mlu_allow_dynamic_smem(outer_update_kernel<true, H>); }) < OB_SMEM)
        return MAGMA_ERR_NOT_SUPPORTED;
    const int K = min(OUTER_NB, min(m, n) - J);
    if (K <= 0 || J + K >= n) return MAGMA_SUCCESS;
    const int tiles = (n - J - K + OB_TN - 1) / OB_TN;
    cudaStream_t s = q->stream;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        MLU_LAUNCH(mlu::KC_OUTER, s, outer_update_kernel<true, H><<<dim3(tiles, nb), OB_THREADS, OB_SMEM, s>>>(
            m, n, J, dA + b0, ldda, ipiv ? ipiv + b0 : nullptr, StepSizes{nullptr, nullptr, nullptr},
            Ub + (size_t)b0 * upad * OUTER_NB, upad));
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}
template magma_int_t outer_prep_tc<__nv_bfloat16>(int, int, int, float **, int, int **, int, __nv_bfloat16 *,
                                                  int, magma_queue_t);
template magma_int_t outer_prep_tc<__half>(int, int, int, float **, int, int **, int, __half *, int,
                                           magma_queue_t);

}  // namespace mlu
