// lu_tc.cu -- FP32 batched LU whose trailing updates run on the 5th-generation
// tensor cores with BF16 or FP16 operands and FP32 accumulation.
//
// The reference's half-precision factorisation (magma_xhsgetrf_gpu,
// src/xhsgetrf_gpu.cpp:212-630) keeps the matrix in FP32, factors the panel
// on the CPU and sends the trailing update to cublasGemmEx with FP16 inputs
// and FP32 accumulation (Magma_PREC_SHT, src/dxgesv_gmres_gpu.cpp:262-266).
// Here the panel, the interchanges and the TRSM are the FP32 kernels of the
// plain path (lu_core.cuh) and the trailing update A22 -= L21 U12 of every
// step whose trailing block is at least 128 x 128 is:
//   tc_stage_kernel   rounds L21 (rows) and U12 (columns) to BF16/FP16 into a
//                     K-major staging buffer [batch][row][32] (K padded with
//                     zeros to 32);
//   tc_update_kernel  one CTA per 128x128 tile: TMA (cp.async.bulk.tensor,
//                     64-byte swizzle) brings the two 8 KB operand tiles into
//                     shared memory, one thread issues two tcgen05.mma
//                     kind::f16 (M=128, N=128, K=16) with the A-negate bit
//                     set, so TMEM receives D = -L21 U12 in FP32, and four
//                     warps read D back with tcgen05.ld and add it to A22.
// Smaller trailing blocks use the FP32 SIMT tile of the plain path.
//
// For matrices the two-level blocking serves (at most 1024 rows, columns right
// of a first 128-column block; lu_blocked.cu, lu_outer.cu) the update is done
// once per 128-column block instead, with K = 128:
//   outer_update_kernel<true, H>  (lu_outer.cu) the block's interchanges and
//                     U12 = L11^{-1} A12 in FP32, in place, and U12 rounded
//                     to H into the staging buffer Ub[batch][row][128];
//   tc_stage_l21_kernel  L21 rounded to H into Lb[batch][row][128];
//   tc_gemm128_kernel  one CTA per 128x128 tile of A22: TMA brings the four
//                     32-deep slices of both operands (64 KB), one thread
//                     issues eight tcgen05.mma kind::f16 (K = 16 each) into
//                     one TMEM accumulator, and four warps add it to A22.
//
// Every wait on an mbarrier is bounded: on timeout the CTA records an error
// in a device flag (the host returns MAGMA_ERR_UNKNOWN), waits once more for
// its own copies, frees its tensor memory and exits.
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <type_traits>

namespace mlu {

constexpr int TC_M = 128, TC_N = 128, TC_K = 32;
constexpr uint32_t TC_TILE_BYTES = TC_M * TC_K * 2;      // 8 KB per operand tile
constexpr long long TC_WAIT_CYCLES = 200ll * 1000 * 1000;  // ~0.1 s at 2 GHz per wait

// ---------------------------------------------------------------------------
// PTX helpers

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes) : "memory");
}

// Wait for phase `parity` of the mbarrier, at most `limit` SM clocks (by
// default TC_WAIT_CYCLES); false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit = TC_WAIT_CYCLES)
{
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    while (clock64() - t0 < limit) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with 64-byte swizzle: rows of 64 bytes (32 half-precision values), 8-row
// groups 512 bytes apart.  Fields: start address >> 4 [0,14), leading byte
// offset >> 4 [16,30) (unused for swizzled K-major, 1), stride byte offset >> 4
// [32,46), descriptor version 1 [46,48), swizzle mode [61,64) (4 = 64-byte).
__device__ __forceinline__ uint64_t kmajor_sw64_desc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// Instruction descriptor of tcgen05.mma kind::f16: D F32 [4,6)=1, A and B
// format [7,10) / [10,13) (0 = F16, 1 = BF16), negate A [13], both K-major,
// N >> 3 at [17,23), M >> 4 at [24,29).
__host__ __device__ constexpr uint32_t f16_idesc(bool bf16)
{
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | (1u << 13) |
           ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

// ---------------------------------------------------------------------------
// Staging: Lb[mat][i][k] = rnd(L21(i,k)), Ub[mat][j][k] = rnd(U12(k,j)), k < 32
// (zero for k >= ib), for i < rm, j < rn.  One thread per (row or column, k).
template <typename H>
__device__ __forceinline__ H to_half(float x);
template <> __device__ __forceinline__ __nv_bfloat16 to_half<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <> __device__ __forceinline__ __half to_half<__half>(float x) { return __float2half_rn(x); }

template <typename H>
__global__ void __launch_bounds__(256)
tc_stage_kernel(int m, int n, int j0, int ib, float **dA_array, int ldda, H *Lb, H *Ub, int pad)
{
    const int mat = blockIdx.y;
    const float *A = dA_array[mat];
    const int rm = m - j0 - ib, rn = n - j0 - ib;
    H *L = Lb + (size_t)mat * pad * TC_K;
    H *U = Ub + (size_t)mat * pad * TC_K;
    const int total = (rm + rn) * TC_K;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        if (e < rm * TC_K) {
            const int i = e % rm, k = e / rm;           // coalesced down a column of L21
            const float v = k < ib ? A[j0 + ib + i + (size_t)(j0 + k) * ldda] : 0.f;
            L[(size_t)i * TC_K + k] = to_half<H>(v);
        } else {
            const int f = e - rm * TC_K;
            const int k = f % TC_K, j = f / TC_K;       // coalesced down a column of U12
            const float v = k < ib ? A[j0 + k + (size_t)(j0 + ib + j) * ldda] : 0.f;
            U[(size_t)j * TC_K + k] = to_half<H>(v);
        }
    }
}

// ---------------------------------------------------------------------------
// One 128x128 tile of A22 += -(L21 U12) on the tensor cores.
template <bool BF16>
__global__ void __launch_bounds__(128, 1)
tc_update_kernel(const __grid_constant__ CUtensorMap tmL, const __grid_constant__ CUtensorMap tmU,
                 float **dA_array, int ldda, int m, int n, int j0, int ib, int tiles_m, int *err)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar_tma, bar_mma;
    __shared__ uint32_t tmem_base;
    // operand tiles on a 1024-byte boundary (64-byte swizzle repeats every 512 bytes)
    unsigned char *sbase = (unsigned char *)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char *sL = sbase, *sU = sbase + TC_TILE_BYTES;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mat = blockIdx.y;
    const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&tmem_base)), "r"(TC_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar_tma, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    __shared__ int s_ok;
    if (tid == 0) {
        mbar_expect_tx(&bar_tma, 2 * TC_TILE_BYTES);
        tma_load_3d(sL, &tmL, 0, tm * TC_M, mat, &bar_tma);
        tma_load_3d(sU, &tmU, 0, tn * TC_N, mat, &bar_tma);
        int ok = mbar_wait(&bar_tma, 0);
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t idesc = f16_idesc(BF16);
            const uint32_t aL = smem_u32(sL), aU = smem_u32(sU);
#pragma unroll
            for (int kk = 0; kk < TC_K / 16; kk++) {
                const uint64_t da = kmajor_sw64_desc(aL + kk * 32);
                const uint64_t db = kmajor_sw64_desc(aU + kk * 32);
                const uint32_t acc = kk > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(smem_u32(&bar_mma)) : "memory");
        } else {
            atomicExch(err, 1);
            mbar_wait(&bar_tma, 0);          // give the copies in flight one more chance
        }
        s_ok = ok;
    }
    __syncthreads();
    const bool ok = s_ok && mbar_wait(&bar_mma, 0);
    if (s_ok && !ok && lane == 0) atomicExch(err, 2);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (ok) {
        // warp w reads TMEM lanes 32w..32w+31: thread = one row of the tile
        float *A = dA_array[mat];
        const int row = warp * 32 + lane;
        const int r = j0 + ib + tm * TC_M + row;
        const int cbase = j0 + ib + tn * TC_N;
#pragma unroll 1
        for (int cc = 0; cc < TC_N; cc += 16) {
            // this chunk's 16 elements of A22 first: all loads in flight together and
            // overlapping the TMEM read (element by element, each load would wait for
            // the previous store)
            float a[16];
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int c = cbase + cc + j;
                a[j] = (r < m && c < n) ? A[r + (size_t)c * ldda] : 0.f;
            }
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                  "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                  "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < m) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = cbase + cc + j;
                    if (c < n) A[r + (size_t)c * ldda] = a[j] + __uint_as_float(v[j]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N));
}

// ---------------------------------------------------------------------------
// Two-level form.  Lb[mat][i][k] = rnd(L(E + i, J + k)) for i < m - E, k < 128
// (zero for k >= K).  One CTA per (matrix, 32 rows): coalesced reads down the
// columns of L21 into shared memory, then rows of 128 k written as pairs.
constexpr int TC_KB = 128;                           // k of the two-level update
template <typename H2, typename H>
__global__ void __launch_bounds__(256)
tc_stage_l21_kernel(int m, int J, int K, float **dA_array, int ldda, H *Lb, int pad)
{
    __shared__ float t[TC_KB][33];
    const int mat = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int E = J + K, r0 = E + blockIdx.x * 32;
    const float *A = dA_array[mat];
    for (int k = warp; k < TC_KB; k += 8)
        t[k][lane] = (k < K && r0 + lane < m) ? A[r0 + lane + (size_t)(J + k) * ldda] : 0.f;
    __syncthreads();
    H *L = Lb + (size_t)mat * pad * TC_KB + (size_t)(r0 - E) * TC_KB;
    for (int x = tid; x < 32 * TC_KB / 2; x += 256) {
        const int row = x / (TC_KB / 2), kp = x % (TC_KB / 2);
        if (r0 + row < m) {
            H2 v;
            v.x = to_half<H>(t[2 * kp][row]);
            v.y = to_half<H>(t[2 * kp + 1][row]);
            *reinterpret_cast<H2 *>(L + (size_t)row * TC_KB + 2 * kp) = v;
        }
    }
}

// One 128x128 tile of A22 (rows and columns from E) += -(L21 U12) with K = 128:
// TMA loads the four 32-deep slices of each operand (64-byte swizzle, 8 KB
// each), one thread issues the eight MMAs, four warps read TMEM back and add.
template <bool BF16>
__global__ void __launch_bounds__(128, 1)
tc_gemm128_kernel(const __grid_constant__ CUtensorMap tmL, const __grid_constant__ CUtensorMap tmU,
                  float **dA_array, int ldda, int m, int n, int E, int tiles_m, int *err)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar_tma, bar_mma;
    __shared__ uint32_t tmem_base;
    __shared__ int s_ok;
    unsigned char *sbase = (unsigned char *)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char *sL = sbase, *sU = sbase + (TC_KB / TC_K) * TC_TILE_BYTES;   // 32 KB each
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mat = blockIdx.y;
    const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&tmem_base)), "r"(TC_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar_tma, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (tid == 0) {
        mbar_expect_tx(&bar_tma, 2 * (TC_KB / TC_K) * TC_TILE_BYTES);
#pragma unroll
        for (int c = 0; c < TC_KB / TC_K; c++) {
            tma_load_3d(sL + c * TC_TILE_BYTES, &tmL, c * TC_K, tm * TC_M, mat, &bar_tma);
            tma_load_3d(sU + c * TC_TILE_BYTES, &tmU, c * TC_K, tn * TC_N, mat, &bar_tma);
        }
        int ok = mbar_wait(&bar_tma, 0);
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t idesc = f16_idesc(BF16);
            const uint32_t aL = smem_u32(sL), aU = smem_u32(sU);
#pragma unroll
            for (int s = 0; s < TC_KB / 16; s++) {
                const uint32_t off = (s >> 1) * TC_TILE_BYTES + (s & 1) * 32;
                const uint64_t da = kmajor_sw64_desc(aL + off);
                const uint64_t db = kmajor_sw64_desc(aU + off);
                const uint32_t acc = s > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(smem_u32(&bar_mma)) : "memory");
        } else {
            atomicExch(err, 1);
            mbar_wait(&bar_tma, 0);          // give the copies in flight one more chance
        }
        s_ok = ok;
    }
    __syncthreads();
    const bool ok = s_ok && mbar_wait(&bar_mma, 0);
    if (s_ok && !ok && lane == 0) atomicExch(err, 2);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (ok) {
        // warp w reads TMEM lanes 32w..32w+31: thread = one row of the tile
        float *A = dA_array[mat];
        const int r = E + tm * TC_M + warp * 32 + lane;
        const int cbase = E + tn * TC_N;
        // the next chunk's 16 elements of A22 are loaded before this chunk is added
        float a[16], an[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int c = cbase + j;
            an[j] = (r < m && c < n) ? A[r + (size_t)c * ldda] : 0.f;
        }
#pragma unroll 1
        for (int cc = 0; cc < TC_N; cc += 16) {
#pragma unroll
            for (int j = 0; j < 16; j++) a[j] = an[j];
            if (cc + 16 < TC_N) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = cbase + cc + 16 + j;
                    an[j] = (r < m && c < n) ? A[r + (size_t)c * ldda] : 0.f;
                }
            }
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                  "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                  "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < m) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = cbase + cc + j;
                    if (c < n) A[r + (size_t)c * ldda] = a[j] + __uint_as_float(v[j]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N));
}

// ---------------------------------------------------------------------------
// Self-test of the bounded waits: one CTA takes tensor memory as the update
// kernel does, then waits on an mbarrier that nothing arrives at (no copy and
// no MMA is ever issued, so nothing is in flight when the wait gives up).  The
// wait runs out after `limit` clocks, the CTA records error code 3, frees its
// tensor memory and returns -- the path every real wait takes on a timeout.
__global__ void __launch_bounds__(128, 1)
tc_wait_selftest_kernel(long long limit, int *err)
{
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&tmem_base)), "r"(32));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    if (tid == 0 && !mbar_wait(&bar, 0, limit)) atomicExch(err, 3);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(32));
}

// ---------------------------------------------------------------------------
// Host side

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        cudaGetLastError();
    }
    return fn;
}

// 3-D map over a staging buffer [batch][pad][kdim] of 16-bit values (kdim 32
// or 128), box 32 x 128 x 1: one 32-deep slice of a 128-row operand tile.
static bool make_map(CUtensorMap *map, void *base, int pad, int batch, bool bf16, int kdim = TC_K)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)kdim, (cuuint64_t)pad, (cuuint64_t)batch};
    const cuuint64_t strides[2] = {(cuuint64_t)kdim * 2, (cuuint64_t)pad * kdim * 2};
    const cuuint32_t box[3] = {(cuuint32_t)TC_K, (cuuint32_t)TC_M, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
                          3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

struct TcLayout {
    int pad;
    size_t lb, ub, err, total;
};

static TcLayout tc_layout(int m, int n, int batch)
{
    TcLayout L;
    L.pad = ((max(m, n) + TC_M - 1) / TC_M) * TC_M;
    // rows of 128 k (the two-level form); the one-level form uses the first 32
    const size_t half_bytes = (size_t)batch * L.pad * TC_KB * 2;
    L.lb = 0;
    L.ub = (half_bytes + 1023) & ~(size_t)1023;
    L.err = L.ub + ((half_bytes + 1023) & ~(size_t)1023);
    L.total = L.err + 256;
    return L;
}

template <typename H, bool BF16>
static magma_int_t tc_getrf(int m, int n, float **dA, int ldda, int **ipiv, int *info, int batch,
                            void *work, magma_queue_t q);

}  // namespace mlu

// panel / swap kernels of the plain path (lu_blocked.cu)
namespace mlu {
template <typename T>
magma_int_t blocked_getrf_steps(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                                magma_queue_t q, int j0, int ib, bool update);
template <typename T>
int blocked_panel_width(int m, int n, int j0);
typedef magma_int_t (*OuterUpdateFn)(int J, void *ctx);
magma_int_t blocked_getrf_two_level(int m, int n, float **dA, int ldda, int **ipiv, int *info,
                                    int batch, magma_queue_t q, OuterUpdateFn outer, void *ctx);
bool two_level_applies(int m, int n);
template <typename H>
magma_int_t outer_prep_tc(int m, int n, int J, float **dA, int ldda, int **ipiv, int batch, H *Ub,
                          int upad, magma_queue_t q);
}

namespace mlu {

// Arguments of the two-level form's update right of a block.
template <typename H>
struct TcOuterCtx {
    int m, n, ldda, batch, pad;
    float **dA;
    int **ipiv;
    H *Lb, *Ub;
    int *err;
    CUtensorMap mapL, mapU;
    magma_queue_t q;
};

template <typename H, bool BF16>
static magma_int_t tc_outer_update(int J, void *vctx)
{
    TcOuterCtx<H> &c = *static_cast<TcOuterCtx<H> *>(vctx);
    const int K = min(TC_KB, min(c.m, c.n) - J), E = J + K;
    magma_int_t rc = outer_prep_tc<H>(c.m, c.n, J, c.dA, c.ldda, c.ipiv, c.batch, c.Ub, c.pad, c.q);
    if (rc != 0 || E >= c.m) return rc;             // no rows below the block: U12 was all
    using H2 = typename std::conditional<BF16, __nv_bfloat162, __half2>::type;
    const int rm = c.m - E, rn = c.n - E;
    const int tiles_m = (rm + TC_M - 1) / TC_M, tiles_n = (rn + TC_N - 1) / TC_N;
    cudaStream_t s = c.q->stream;
    MLU_LAUNCH(mlu::KC_OTHER, s, tc_stage_l21_kernel<H2, H><<<dim3((rm + 31) / 32, c.batch), 256, 0, s>>>(
        c.m, J, K, c.dA, c.ldda, c.Lb, c.pad));
    // 2 x 32 KB of operands + alignment, requested as 66 KB so that at most three
    // CTAs share an SM: three 128-column accumulators within its 512 TMEM columns
    MLU_LAUNCH(mlu::KC_TC_UPDATE, s, tc_gemm128_kernel<BF16><<<dim3(tiles_m * tiles_n, c.batch), 128, 66 * 1024, s>>>(
        c.mapL, c.mapU, c.dA, c.ldda, c.m, c.n, E, tiles_m, c.err));
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

template <typename H, bool BF16>
static magma_int_t tc_getrf(int m, int n, float **dA, int ldda, int **ipiv, int *info, int batch,
                            void *work, magma_queue_t q)
{
    const TcLayout L = tc_layout(m, n, batch);
    if (two_level_applies(m, n) && batch <= MLU_MAX_GRID_Y) {
        // 128-column blocks, one K = 128 tensor-core update right of each
        char *w = (char *)work;
        TcOuterCtx<H> c;
        c.m = m; c.n = n; c.ldda = ldda; c.batch = batch; c.pad = L.pad;
        c.dA = dA; c.ipiv = ipiv; c.q = q;
        c.Lb = (H *)(w + L.lb);
        c.Ub = (H *)(w + L.ub);
        c.err = (int *)(w + L.err);
        if (!make_map(&c.mapL, c.Lb, L.pad, batch, BF16, TC_KB) ||
            !make_map(&c.mapU, c.Ub, L.pad, batch, BF16, TC_KB))
            return MAGMA_ERR_NOT_SUPPORTED;
        static size_t dyn_cache[MLU_MAX_DEVICES];
        if (mlu_device_cached(dyn_cache, [] { return mlu_allow_dynamic_smem(tc_gemm128_kernel<BF16>); }) <
            66 * 1024)
            return MAGMA_ERR_NOT_SUPPORTED;
        cudaMemsetAsync(c.err, 0, sizeof(int), q->stream);
        return blocked_getrf_two_level(m, n, dA, ldda, ipiv, info, batch, q, tc_outer_update<H, BF16>, &c);
    }
    char *w = (char *)work;
    H *Lb = (H *)(w + L.lb);
    H *Ub = (H *)(w + L.ub);
    int *err = (int *)(w + L.err);
    CUtensorMap mapL, mapU;
    if (!make_map(&mapL, Lb, L.pad, batch, BF16) || !make_map(&mapU, Ub, L.pad, batch, BF16))
        return MAGMA_ERR_NOT_SUPPORTED;
    static size_t dyn_cache[MLU_MAX_DEVICES];
    const size_t dyn = mlu_device_cached(dyn_cache, [] { return mlu_allow_dynamic_smem(tc_update_kernel<BF16>); });
    // 2 x 8 KB of operands + alignment, requested as 56 KB so that at most four
    // CTAs share an SM: four 128-column accumulators fill its 512 TMEM columns
    const size_t smem = 56 * 1024;
    if (smem > dyn) return MAGMA_ERR_NOT_SUPPORTED;
    if (batch > MLU_MAX_GRID_Y) return MAGMA_ERR_NOT_SUPPORTED;
    cudaMemsetAsync(err, 0, sizeof(int), q->stream);
    const int mn = min(m, n);
    for (int j0 = 0; j0 < mn;) {
        // panel + interchanges + TRSM; the trailing update only when it is small
        const int ib = blocked_panel_width<float>(m, n, j0);
        const int rm = m - j0 - ib, rn = n - j0 - ib;
        const bool use_tc = rm >= TC_M && rn >= TC_N;
        magma_int_t rc = blocked_getrf_steps<float>(m, n, dA, ldda, ipiv, info, batch, q, j0, ib,
                                                    !use_tc);
        if (rc != 0) return rc;
        if (use_tc) {
            const int tiles_m = (rm + TC_M - 1) / TC_M, tiles_n = (rn + TC_N - 1) / TC_N;
            for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
                const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
                const int blocks = min(64, ((rm + rn) * TC_K + 255) / 256);
                MLU_LAUNCH(mlu::KC_OTHER, q->stream, tc_stage_kernel<H><<<dim3(blocks, nb), 256, 0, q->stream>>>(
                    m, n, j0, ib, dA + b0, ldda, Lb + (size_t)b0 * L.pad * TC_K,
                    Ub + (size_t)b0 * L.pad * TC_K, L.pad));
            }
            MLU_LAUNCH(mlu::KC_TC_UPDATE, q->stream, tc_update_kernel<BF16><<<dim3(tiles_m * tiles_n, batch), 128, smem, q->stream>>>(
                mapL, mapU, dA, ldda, m, n, j0, ib, tiles_m, err));
        }
        j0 += ib;
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

}  // namespace mlu

using namespace mlu;

extern "C" magma_int_t magma_sgetrf_batched_tc(magma_int_t precision, magma_int_t m, magma_int_t n,
                                               float **dA_array, magma_int_t ldda,
                                               magma_int_t **ipiv_array, magma_int_t *info_array,
                                               void *work, size_t *lwork, magma_int_t batchCount,
                                               magma_queue_t queue)
{
    magma_int_t arginfo = 0;
    if (precision != 905 && precision != 930) arginfo = -1;
    else if (m < 0) arginfo = -2;
    else if (n < 0) arginfo = -3;
    else if (ldda < mlu_max(1, m)) arginfo = -5;
    if (arginfo != 0) {
        magma_xerbla(__func__, -arginfo);
        return arginfo;
    }
    const TcLayout L = tc_layout(m, n, mlu_max(batchCount, 0));
    if (work == nullptr) {
        *lwork = L.total;
        return 0;
    }
    if (*lwork < L.total) return -9;
    if (m == 0 || n == 0 || batchCount <= 0) return 0;
    magma_int_t rc = precision == 930
                         ? tc_getrf<__nv_bfloat16, true>(m, n, dA_array, ldda, ipiv_array, info_array,
                                                         batchCount, work, queue)
                         : tc_getrf<__half, false>(m, n, dA_array, ldda, ipiv_array, info_array,
                                                   batchCount, work, queue);
    return rc;
}

// Runs tc_wait_selftest_kernel with a wait limit of `limit_cycles` SM clocks
// (1 .. 4e9) and returns the error code it recorded (3 when the wait ran out,
// as it must), or a negative MAGMA error.  `flag`: one int of device memory.
// Synchronises the queue.
extern "C" magma_int_t magma_sgetrf_batched_tc_wait_selftest(long long limit_cycles, magma_int_t *flag,
                                                             magma_queue_t queue)
{
    if (limit_cycles < 1 || limit_cycles > 4000000000ll) return -1;
    if (flag == nullptr) return -2;
    cudaMemsetAsync(flag, 0, sizeof(int), queue->stream);
    MLU_LAUNCH(mlu::KC_OTHER, queue->stream,
               tc_wait_selftest_kernel<<<1, 128, 0, queue->stream>>>(limit_cycles, flag));
    MLU_CHECK_LAUNCH();
    int e = 0;
    cudaMemcpyAsync(&e, flag, sizeof(int), cudaMemcpyDeviceToHost, queue->stream);
    if (cudaStreamSynchronize(queue->stream) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    return e;
}

// Error flag of the last magma_sgetrf_batched_tc on this workspace (0 = fine);
// synchronises the queue.
extern "C" magma_int_t magma_sgetrf_batched_tc_status(magma_int_t m, magma_int_t n, void *work,
                                                      magma_int_t batchCount, magma_queue_t queue)
{
    const TcLayout L = tc_layout(m, n, mlu_max(batchCount, 0));
    int e = 0;
    cudaMemcpyAsync(&e, (char *)work + L.err, sizeof(int), cudaMemcpyDeviceToHost, queue->stream);
    if (cudaStreamSynchronize(queue->stream) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    return e;
}
